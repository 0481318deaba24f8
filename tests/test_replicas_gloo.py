"""The multi-GPU form is replicas: every rank applies the operator to its
own columns and the ranks only meet for timing.  This checks that
bookkeeping (barrier, max over ranks, whole-job throughput) with two gloo
ranks on the CPU."""

import os
import socket

import pytest

torch = pytest.importorskip('torch')
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))))
    import bench
    r, w, local = bench.dist_info()
    barrier, allmax = bench._dist_setup(torch, w, local, backend='gloo')
    barrier()
    # each replica "took" a different time; the job time is the slowest
    t = allmax(1.0 + r)
    out[rank] = t
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_take_max_time():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world,
             join=True)
    assert out[0] == out[1] == 2.0


def test_batched_specs_are_per_rank_and_reproducible():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))))
    import bench
    a, b = bench.batched_specs(seed=0), bench.batched_specs(seed=0)
    c = bench.batched_specs(seed=1)
    assert [(k, n, m) for k, n, m, _ in a] == [(k, n, m) for k, n, m, _ in b]
    assert [(k, n, m) for k, n, m, _ in a] != [(k, n, m) for k, n, m, _ in c]
    assert len(a) == 512 and all(64 <= n <= 65536 for _, n, _, _ in a)
