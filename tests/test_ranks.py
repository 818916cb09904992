"""The N-GPU path of bench.py on CPU: N replicas of one index, each searching
its own queries, with the job timed as the slowest rank. Two `gloo` ranks
check the collectives the timing and the setting choice go through; the data
rule (same index on every rank, different queries) and the reference arm's
idle ranks are checked in one process."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's own elapsed time; the job is as slow as its slowest rank
        slowest = bench.max_over_ranks(dist, 10.0 + 2.5 * rank)
        # each rank's sweep picks a setting; all of them run rank 0's
        choice = bench.from_rank0(dist, 17 if rank == 0 else 4 + rank)
        out.put((rank, slowest, choice))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_slowest_rank_and_rank0_setting(world):
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == list(range(world))
    assert all(g[1] == 10.0 + 2.5 * (world - 1) for g in got)
    assert all(g[2] == 17 for g in got)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(None, 3.25) == 3.25
    assert bench.from_rank0(None, 9) == 9


def test_replicas_share_the_index_not_the_queries():
    torch = pytest.importorskip("torch")
    import bench
    kw = dict(n=600, d=32, ncomp=12, seed=5, queries=16, train_queries=8, dev="cpu")
    b0, q0, t0 = bench.make_data(torch, **kw, qseed=bench.query_seed(5, 0))
    b1, q1, t1 = bench.make_data(torch, **kw, qseed=bench.query_seed(5, 1))
    bd, qd, _ = bench.make_data(torch, **kw)
    assert torch.equal(b0, b1) and torch.equal(t0, t1)   # one index, one probe model's data
    assert not torch.equal(q0, q1)                        # each replica its own queries
    assert torch.equal(b0, bd) and torch.equal(q0, qd)    # rank 0 = the single-GPU run
    assert np.allclose(q1.norm(dim=1).numpy(), 1.0, atol=1e-5)
    seeds = {bench.query_seed(5, r) for r in range(8)}
    assert len(seeds) == 8


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.main() is None
    assert capsys.readouterr().out == ""
