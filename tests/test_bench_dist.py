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

    def fake_one_run(engine, e2e, batch=None, collect=False):
        together.wait()
        seen[engine] = (threading.current_thread() is not threading.main_thread(), e2e, batch, collect)
        return 10 * engine, engine, ({"engine": engine} if collect else None)

    monkeypatch.setattr(bench, "one_run", fake_one_run)
    assert bench.step([1, 2, 3], True, 8) == (60, 6, None)
    assert sorted(seen) == [1, 2, 3]
    assert all(v == (True, True, 8, False) for v in seen.values())
    # outputs are collected from the first engine only
    assert bench.step([1, 2, 3], False, 8, collect=True)[2] == {"engine": 1}
    assert [seen[k][3] for k in (1, 2, 3)] == [True, False, False]

    def failing(engine, e2e, batch=None, collect=False):
        if engine == 2:
            raise RuntimeError("engine 2 failed")
        return 0, 0, None

    monkeypatch.setattr(bench, "one_run", failing)
    with pytest.raises(RuntimeError, match="engine 2 failed"):
        bench.step([1, 2, 3], False)


def test_error_comparison_reports_worst_site():
    """bench._compare: largest eigenvalue error, its site, the error over the
    parity tolerance, spectral / entropy / C(T) errors."""
    import sys
    import numpy as np
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    bench.select_workload("siam_fdm_nk1024")
    ref = [np.linspace(0, 1, 5), np.linspace(0, 2, 7)]
    got = {"eig": [ref[0].copy(), ref[1] + 3e-10], "spectra": [np.array([1.0, 2.0])],
           "entropy": np.array([0.5, 0.25]), "cv": np.array([1.0, 2.0])}
    T = np.array([1e-8, 1e-3])
    r = bench._compare(got, ref, [np.array([1.0, 2.0 + 2e-7])], np.array([0.5, 0.25]), np.array([5.0, 2.0]), T)
    assert r["eig_max_abs_site"] == 1 and abs(r["eig_max_abs"] - 3e-10) < 1e-15
    assert abs(r["eig_max_over_tol"] - 3.0) < 1e-4
    assert abs(r["spectral_max_rel"] - 1e-7) < 1e-12
    assert r["entropy_max_abs"] == 0.0
    assert r["cv_max_rel_T_ge_2.6e-7"] == 0.0  # the T=1e-8 point is outside the compared range
    got["eig"][1] = got["eig"][1][:3]
    assert bench._compare(got, ref, [], got["entropy"], got["cv"], T) == {"eig_count_mismatch_at_site": 1}
