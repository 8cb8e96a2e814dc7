"""Multi-process (world_size 2, gloo, CPU) checks of bench.py's replica
logic: the timing reduction is the maximum over ranks, the value aggregates
all ranks' nodes, and the reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_local = 0.5 + rank  # rank 1 is the slow one
    t = bench.max_over_ranks(t_local, world, "cpu")
    out[rank] = (t, bench.aggregate_nodes_per_s(world, bench.M_NODES, 10, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_aggregate_gloo():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    import bench
    for rank in range(world):
        t, v = res[rank]
        assert t == 1.5
        assert v == pytest.approx(world * bench.M_NODES * 10 / 1.5)


def test_reference_arm_only_on_rank0(monkeypatch):
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2

    monkeypatch.setenv("RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_reference_run", lambda *a, **k: called.append(1))
    assert bench.run_reference(A()) == 0
    assert not called
