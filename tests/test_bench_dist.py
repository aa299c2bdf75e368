"""The multi-rank reduction of bench.py (max over ranks of the timed sums),
exercised with two gloo ranks on the CPU."""
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


def _rank(rank, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        assert bench._dist() == (2, rank)
        out[rank] = bench.max_over_ranks([1.0 + rank, 10.0 - rank, -3.0])
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(port, out), nprocs=2, join=True)
        assert out[0] == out[1] == [2.0, 10.0, -3.0]


def test_max_over_ranks_without_process_group():
    import bench
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]


def test_step_runs_every_engine_on_its_own_thread(monkeypatch):
    """bench.step drives each engine from its own host thread, sums the
    per-engine input / output byte counts and re-raises a failure."""
    import sys
    import threading
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    seen = {}
    together = threading.Barrier(3, timeout=30)  # passes only if all three run at once

    def fake_one_run(engine, e2e, batch=None):
        together.wait()
        seen[engine] = (threading.current_thread() is not threading.main_thread(), e2e, batch)
        return 10 * engine, engine

    monkeypatch.setattr(bench, "one_run", fake_one_run)
    assert bench.step([1, 2, 3], True, 8) == (60, 6)
    assert sorted(seen) == [1, 2, 3]
    assert all(v == (True, True, 8) for v in seen.values())

    def failing(engine, e2e, batch=None):
        if engine == 2:
            raise RuntimeError("engine 2 failed")
        return 0, 0

    monkeypatch.setattr(bench, "one_run", failing)
    with pytest.raises(RuntimeError, match="engine 2 failed"):
        bench.step([1, 2, 3], False)
