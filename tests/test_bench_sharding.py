"""The bench's multi-rank path on the host (two gloo ranks on CPU): under
torchrun every rank steps its own draw of the workload (world-sharded, no
collective on the data path) and the reported value is the units all ranks
processed over the slowest rank's time.  The GPU legs need a device; the
sharding and the reductions around them do not."""
import multiprocessing as mp
import os
import socket
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    from constraintphysics_gb300 import scenes
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        r, n, _ = bench.dist_env()
        scs = scenes.batched_worlds(seed=bench.shard_seed(0, r), n_worlds=6)
        units = bench.dynamic_bodies(scs)
        ms = 10.0 + 5.0 * r   # the ranks' timed regions differ
        (ms_max,), (units_all,) = bench.across_ranks(n, [ms], [units])
        q.put((r, units, ms_max, units_all, [sc.name for sc in scs]))
    finally:
        dist.destroy_process_group()


def test_ranks_shard_the_worlds_and_reduce_max_time_and_total_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, u0, m0, t0, n0), (r1, u1, m1, t1, n1) = got
    assert (r0, r1) == (0, 1)
    assert m0 == m1 == 15.0                      # the slowest rank's time, on every rank
    assert t0 == t1 == u0 + u1                   # the units of all ranks
    assert n0 != n1                              # each rank draws its own worlds


def test_one_rank_reduces_to_itself():
    sys.path.insert(0, REPO)
    import bench
    assert bench.across_ranks(1, [3.0, 4.0], [7]) == ([3.0, 4.0], [7.0])
    assert bench.shard_seed(5, 0) == 5 and bench.shard_seed(5, 2) == 2005
