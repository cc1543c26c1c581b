"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas only).

bench.py under torchrun runs one independent solve per rank: no data-path
collective, a barrier around the timed region and a MAX all-reduce of the
timed totals; rank 0 prints the JSON line, the others exit 0.  These tests
run that host logic as two spawned processes with the gloo backend on
127.0.0.1 (no GPU).
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, totals, out_q):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench

    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_env()
        dist.barrier()
        total, value = bench.aggregate_ranks(torch, ws, totals[rank], nodes=1000, steps=10, device="cpu")
        e2e, _ = bench.aggregate_ranks(torch, ws, 2.0 * totals[rank], nodes=1000, steps=1, device="cpu")
        dist.barrier()
        out_q.put((rank, got_ws, got_rank, got_local, total, value, e2e))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp

    ws, port = 2, _free_port()
    totals = [10.0, 15.0]  # ms of the timed region per rank
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, totals, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got_ws, got_rank, got_local, total, value, e2e in res:
        assert (got_ws, got_rank, got_local) == (ws, rank, rank)
        assert total == 15.0  # MAX over ranks
        assert value == pytest.approx(ws * 1000 * 10 / 15e-3)  # whole-job node updates / s
        assert e2e == 30.0


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    # rank 1 returns before touching the oracle or any device
    assert bench.run_reference(None) == 0


def test_single_rank_aggregation_is_local():
    sys.path.insert(0, ROOT)
    import torch
    import bench

    total, value = bench.aggregate_ranks(torch, 1, 20.0, nodes=512000, steps=50)
    assert total == 20.0 and value == pytest.approx(512000 * 50 / 20e-3)
