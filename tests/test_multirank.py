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
