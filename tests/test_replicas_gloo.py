"""The multi-GPU path is replicas only (no collective on the data path): the
per-rank timing reduction and the whole-job rate, run as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "proland-4.0_gb300")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    sys.path.insert(0, PKG)
    import torch.distributed as dist
    from proland_gb300 import replicas
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank                       # rank 1 is the slower replica
    m = replicas.max_over_ranks(ms, dist)
    rate = replicas.whole_job_rate(4096, m, world)
    out[rank] = (m, rate, replicas.rank_seed(2024, rank))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == pytest.approx(2 * 4096 / 0.015)
    assert res[0][2] != res[1][2]


def test_single_process_has_no_group():
    sys.path.insert(0, PKG)
    from proland_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.whole_job_rate(100, 10.0, 1) == pytest.approx(10000.0)
