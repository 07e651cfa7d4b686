"""bench.py's multi-rank path on the CPU: two gloo ranks, as torchrun would
start them.  Each rank takes its own seeds (weak scaling: the runs are
independent, so no data-path collective), and the timed value is the
maximum over ranks (the one collective)."""
import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path[:0] = [str(REPO), str(REPO / "deac-cpp_gb300")]
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        headline = [cfg.seed for cfg, *_ in bench.run_specs(rank, 4)]
        single = [cfg.seed for cfg, *_ in bench.config1_specs(rank)]
        slowest = bench.barrier_max(1.5 + rank, world, "cpu")
        out.put((rank, headline, single, slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_their_own_seeds_and_report_the_slowest():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in procs:
        rank, headline, single, slowest = out.get(timeout=120)
        got[rank] = (headline, single, slowest)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (h0, s0, m0), (h1, s1, m1) = got[0], got[1]
    assert h0 == [1, 2, 3, 4] and h1 == [1025, 1026, 1027, 1028]  # RUNS_PER_GPU seeds per rank
    assert not set(s0) & set(s1)
    assert m0 == m1 == 2.5
