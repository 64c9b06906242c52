"""Replica bookkeeping across ranks (gloo, world size 2, CPU): the timed
region's barrier and the max-over-ranks timing that whole-job throughput is
computed from.  No GPU: the replicas exchange no data."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(r, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(r),
                      LOCAL_RANK=str(r))
    from voxelfragmentml_gb300 import replicas as R
    assert R.init() == 2 and R.rank() == r
    R.barrier()
    ms = 10.0 if r == 0 else 25.0          # rank 1 is the slower replica
    got_max = R.max_over_ranks(ms)
    rate = R.aggregate_rate(1000.0, ms)   # 1000 units per rank
    R.finalize()
    q.put((r, got_max, rate))


def test_two_replicas_max_timing_and_aggregate_rate():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, mx, rate in out:
        assert mx == 25.0                      # every rank sees the slowest time
        assert rate == pytest.approx(2000.0 / 0.025)  # all units / slowest time


def test_single_process_is_a_world_of_one(monkeypatch):
    for k in ("WORLD_SIZE", "RANK"):
        monkeypatch.delenv(k, raising=False)
    from voxelfragmentml_gb300 import replicas as R
    assert R.init() == 1 and R.rank() == 0
    assert R.max_over_ranks(3.5) == 3.5
    assert R.aggregate_rate(100.0, 50.0) == pytest.approx(2000.0)
