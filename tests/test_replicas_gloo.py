"""The multi-GPU bookkeeping of bench.py (ohao_engine_gb300.replicas) with two
gloo ranks on the CPU: barrier, the slowest rank's time on every rank, and
the whole-job rate over it. The path has no exchange step, so this is all
the ranks share."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from ohao_engine_gb300 import replicas
    r = replicas.init("gloo")
    assert (r.world, r.rank) == (world, rank)
    replicas.barrier(r)
    seconds = 1.0 + rank            # rank 1 is the slow one
    mx = replicas.max_over_ranks(r, seconds)
    rate = replicas.whole_job_rate(1000.0, r, seconds)
    out.put((rank, mx, rate))
    replicas.finish(r)


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, out)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, mx, rate in res:
        assert mx == 2.0                      # the slowest rank's time on every rank
        assert rate == pytest.approx(1000.0 * 2 / 2.0)


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from ohao_engine_gb300 import replicas
    r = replicas.init("gloo")
    assert r.world == 1 and r.dist is None
    assert replicas.max_over_ranks(r, 3.5) == 3.5
    assert replicas.whole_job_rate(10.0, r, 2.0) == 5.0
