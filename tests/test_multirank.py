"""The multi-GPU form of the benchmark is independent replicas ("replicas
only": the single-device factorization has no exchange step).  Its only
cross-rank logic is the timing reduction: the job's time is the slowest
rank's, and the job's rate is every rank's units over that time.  Checked
here with two gloo ranks on the CPU."""
import importlib.util
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        b = _bench()
        t = 1.0 + rank                      # rank r took 1 + r seconds
        out[rank] = (b.max_over_ranks(t, dist, "cpu"), b.job_rate(10.0, t, dist, "cpu"))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_timing_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        slowest, rate = res[r]
        assert slowest == 2.0             # the slower rank's time on every rank
        assert rate == pytest.approx(2 * 10.0 / 2.0)


def test_single_process_needs_no_group():
    b = _bench()
    assert b.max_over_ranks(3.5, None) == 3.5
    assert b.job_rate(7.0, 2.0, None) == 3.5
