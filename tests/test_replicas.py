"""The multi-GPU form of the benchmark is replicas: one independent graph per rank, no data
exchange on the path.  The whole-job figure sums the units every rank processed and divides by
the slowest rank's time.  Checked here with two gloo ranks on CPU (no GPU involved)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = 1000.0 * (rank + 1)      # ranks may process different amounts
        ms = 10.0 + 5.0 * rank           # rank 1 is the slowest
        q.put((rank, bench.combine_ranks(units, ms, dist, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_combine_ranks_sums_units_and_takes_slowest_time():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert out[r] == (3000.0, 15.0)


def test_single_process_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(123.0, 4.5, None) == (123.0, 4.5)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        workload, scale, seed, steps, warmup = "cc", 8, 1, 1, 3
    bench.run_reference(A())  # rank 1: returns before any work
    assert capsys.readouterr().out == ""


def test_batch_graphs_split_over_ranks():
    """Under torchrun the batch's graphs are split over the ranks, longest first to the least
    loaded rank: every graph exactly once, loads within one graph of each other."""
    sys.path.insert(0, ROOT)
    import bench
    edges = [5, 100, 7, 100, 3, 60, 60, 1]
    for world in (1, 2, 3, 4):
        parts = bench.assign_graphs(edges, world)
        assert sorted(i for p in parts for i in p) == list(range(len(edges)))
        loads = [sum(edges[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(edges)
    assert bench.assign_graphs(edges, 2) == bench.assign_graphs(edges, 2)


def _batch_rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        edges = [g.num_edges for _, g in bench.batch_graphs(1)]
        mine = bench.assign_graphs(edges, world)[rank]
        units = float(sum(edges[i] for i in mine))
        q.put((rank, mine, bench.combine_ranks(units, 1.0 + rank, dist, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_batch_split_covers_the_batch_with_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {r: (m, c) for r, m, c in (q.get(timeout=300) for _ in procs)}
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(out[0][0] + out[1][0]) == list(range(32))
    assert not set(out[0][0]) & set(out[1][0])
    sys.path.insert(0, ROOT)
    import bench
    total = float(sum(g.num_edges for _, g in bench.batch_graphs(1)))
    assert out[0][1] == out[1][1] == (total, 2.0)
