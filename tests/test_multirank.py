"""Host logic of the multi-GPU bench (replicas, one twist per rank) with world_size 2 on
CPU over gloo: distinct twists per rank, and the reported time is the slowest rank's."""
import importlib.util
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.join(os.path.dirname(__file__), "..")


def _bench():
    spec = importlib.util.spec_from_file_location("ccx_bench", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        out[rank] = (b.max_over_ranks(ms, dist, "cpu"), b.replica_theta(rank))
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replicas_gloo_world2():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] != res[1][1]
    assert res[0][1] == (0.0, 0.0, 0.0)


def test_single_process_needs_no_collective():
    b = _bench()
    assert b.max_over_ranks(3.5, None, "cpu") == 3.5
