"""The replica-parallel bench path (--gpus N) on CPU: world_size 2 over gloo.
Instances are independent, so ranks only meet at the timing barrier and the
max-over-ranks reduction; the job's throughput is all ranks' site-updates over
the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, local = bench.dist_setup(0)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(w)
    t = 1.0 + rank  # rank 1 is the slower replica
    out[rank] = bench.job_throughput(100.0, t, w)
    out[2 + rank] = bench.max_over_ranks(t, w)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_replicas_on_gloo():
    world = 2
    out = mp.get_context("spawn").Array("d", 4)
    port = _free_port()
    procs = [mp.get_context("spawn").Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert list(out[2:]) == [2.0, 2.0]            # both ranks see the slowest time
    assert list(out[:2]) == [100.0, 100.0]        # 2 ranks x 100 units / 2 s


def _sweep_worker(rank, world, port, ok):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import numpy as np
    import torch.distributed as dist
    from trophic_maelstorm_gb300 import api
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seen = []

    def fake_block(ctx, indices, avals, *args):
        # stands in for the GPU batch of this rank's control values
        seen.extend(indices)
        return {ia: (np.full((3, 8), float(ia)), np.full(4, ia, np.uint32)) for ia in indices}

    api._sweep_block = fake_block
    rows, st = api.critical_exp_delta(np.ones(16), 7, 10.0, 0.5, 0.6, 2.0, 1.0, 1.0, 0.1, 1.0, 4, 4,
                                      ctx=object(), distributed=True)
    good = seen == api.shard_indices(7, rank, world)
    if rank == 0:
        good = good and np.array_equal(rows[:, 0], np.repeat(np.arange(7.0), 3))
        good = good and np.array_equal(st, np.repeat(np.arange(7), 4).astype(np.uint32))
    else:
        good = good and rows is None and st is None
    ok[rank] = 1 if good else 0
    dist.destroy_process_group()


def test_sharded_sweep_gathers_rows_on_rank0():
    """critical_exp_delta(distributed=True) on 2 gloo ranks: each rank runs its contiguous
    block of a-values, rank 0 receives every row in a order."""
    world = 2
    ctx = mp.get_context("spawn")
    ok = ctx.Array("i", world)
    port = _free_port()
    procs = [ctx.Process(target=_sweep_worker, args=(r, world, port, ok)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert list(ok) == [1, 1]


@pytest.mark.parametrize("n,world", [(7, 2), (16, 3), (2, 4), (0, 2), (5, 1)])
def test_shard_indices_cover_every_value_once(n, world):
    from trophic_maelstorm_gb300 import api
    parts = [api.shard_indices(n, r, world) for r in range(world)]
    flat = [i for p in parts for i in p]
    assert flat == list(range(n))
    assert max(map(len, parts)) - min(map(len, parts)) <= 1
