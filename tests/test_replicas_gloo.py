"""The replicas path of bench.py on CPU: two gloo ranks, the job time is the
maximum over ranks and the value counts every rank's work (no GPU)."""
import os
import socket

import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    t_local = [2.0, 3.5][rank]
    t_max, value = bench.job_throughput(t_local, 1000.0, world, dist, 'cpu')
    out[rank] = (t_max, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    port = _free_port()
    with mp.get_context('spawn').Manager() as m:   # no fork of a multi-threaded parent
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (3.5, 2 * 1000.0 / 3.5)


def test_single_replica_without_process_group():
    import bench
    assert bench.job_throughput(2.0, 10.0, 1) == (2.0, 5.0)
