"""Serving loop (nrg_server_*): continuous batching of whole runs.

A run served alone, served in a mix with runs that arrive before and while it
is on the GPU, and driven directly through the per-run API must give the same
results: eigenvalues and entropy bit for bit (every kernel on that path sums
in a fixed order), FDM weights to 1e-12 relative (the binning adds with
floating-point atomics, so their order may differ between runs)."""
import math
import threading
import time

import numpy as np
import pytest

from nrgplusplus_gb300 import api, workloads
from nrgplusplus_gb300 import models as M

pytestmark = pytest.mark.gpu

NK, NS, LAM = 96, 14, 2.0


def _req(eps=-0.4, U=0.8, V=0.15, nkeep=NK, nsites=NS):
    return workloads.siam_request(nkeep, nsites, LAM, V, eps=eps, U=U, fdm=True, thermo=True)


def _same(a, b):
    assert len(a["eig"]) == len(b["eig"])
    for x, y in zip(a["eig"], b["eig"]):
        assert np.array_equal(x, y)
    assert np.array_equal(a["entropy"], b["entropy"])
    assert np.array_equal(a["specificHeat"], b["specificHeat"])
    for k in ("GreenFnPositiveWeight", "GreenFnNegativeWeight"):
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-300)


def _direct(engine, eps=-0.4, U=0.8, V=0.15):
    """The same run through the per-run API, in the order the bench drives it:
    V site, Wilson sites with operator update and snapshots, then one backward
    loop feeding the FDM spectrum and the thermodynamics shell by shell."""
    imp, bath = workloads.build_models("siam", eps, U)
    run = api.NrgCore(engine, imp, bath, NK)
    data = api.NrgData(run)
    run.add_bath_site([V, V], 1.0)
    ops = api.OperatorSet(run, M.d_dag_chi())
    api.update_system_operator(run, ops)
    run.update_internal_state()
    eig, min_it = [run.all_eigenvalue], 0
    for it in range(NS):
        h = M.hopping(it, LAM)
        run.add_bath_site([h, h], math.sqrt(LAM) if it > 0 else 1.0)
        api.update_system_operator(run, ops)
        if run.checkHigherEnergyDiscarded():
            data.saveCurrentData(ops)
        else:
            min_it += 1
        run.update_internal_state()
        eig.append(run.all_eigenvalue)
    f = api.FdmSpectrum(run, 2)
    th = api.FdmThermodynamics(run, workloads.temperature_grid())
    cnt = run.nrg_iterations_cnt
    for it in range(NS, min_it, -1):
        cnt -= 1
        data.loadCurrentData(cnt)
        f.calcSpectrum(LAM ** (-(it - 1.0) / 2.0))
        th.calcThermodynamics(LAM ** (-(it - 1.0) / 2.0))
    out = {"eig": eig, **f.saveFinalData(), **th.saveFinalData()}
    f.close()
    th.close()
    ops.close()
    run.close()
    return out


def test_served_run_matches_direct_api(mixed_engine):
    direct = _direct(mixed_engine)
    eng = api.Engine(api.PREC_MIXED)
    srv = api.Server(eng, max_active=4)
    rid = srv.submit(**_req())
    assert srv.wait(rid)
    got = srv.result(rid)
    srv.close()
    eng.close()
    assert len(got["eig"]) == NS + 1
    _same(got, direct)


def test_alone_and_in_mix_are_equal():
    eng = api.Engine(api.PREC_MIXED)
    srv = api.Server(eng, max_active=1)
    rid = srv.submit(**_req())
    assert srv.wait(rid)
    alone = srv.result(rid)
    srv.close()

    srv = api.Server(eng, max_active=8)
    others = [dict(eps=-0.3, U=0.6), dict(eps=-0.5, U=1.0, nkeep=128), dict(V=0.1, nsites=10),
              dict(eps=-0.2, U=0.4, nkeep=64)]
    ids = [srv.submit(**_req(**o)) for o in others]
    target = srv.submit(**_req())
    late = []

    def arrive_late():  # requests that arrive while the mix is on the GPU
        time.sleep(0.3)
        late.append(srv.submit(**_req(eps=-0.35, U=0.7, nsites=12)))
        late.append(srv.submit(**_req(V=0.2, nkeep=80)))

    th = threading.Thread(target=arrive_late)
    th.start()
    assert srv.wait(target)
    mixed = srv.result(target)
    th.join()
    for i in ids + late:
        assert srv.wait(i)
        r = srv.result(i)
        assert np.isfinite(r["entropy"]).all()
    st = srv.stats()
    srv.close()
    eng.close()
    assert st["completed"] == len(others) + 3 and st["failed"] == 0
    assert st["max_active_seen"] > 1  # the runs really shared ticks
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"]
    _same(mixed, alone)


def test_admission_respects_the_budget():
    eng = api.Engine(api.PREC_MIXED)
    nk, ns = 64, 10
    one = 2.0 * ns * (4 * nk) ** 2  # the server's initial estimate for one run
    srv = api.Server(eng, max_active=8, hbm_budget_bytes=int(2.5 * one))
    ids = [srv.submit(**workloads.siam_request(nk, ns - 1, LAM, 0.15, eps=-0.3 - 0.05 * k, U=0.6))
           for k in range(5)]
    for i in ids:
        assert srv.wait(i)
        srv.result(i)
    st = srv.stats()
    srv.close()
    eng.close()
    assert st["completed"] == 5
    assert 1 <= st["max_active_seen"] <= 2


def test_bad_requests_fail_alone():
    eng = api.Engine(api.PREC_MIXED)
    srv = api.Server(eng, max_active=4)
    with pytest.raises(api.NrgError):  # FDM without tracked operators
        srv.submit(**{**_req(), "ops": None})
    bad = _req()
    bad["t"] = np.hstack([bad["t"], bad["t"][:, :1]])  # 3 hoppings for a 2-operator model
    rb = srv.submit(**bad)
    good = srv.submit(**_req(nsites=8))
    assert srv.wait(rb) and srv.wait(good)
    with pytest.raises(api.NrgError) as ei:
        srv.result(rb)
    assert "t_hopping" in str(ei.value)
    assert math.isfinite(srv.result(good)["entropy"][0])
    srv.close()
    eng.close()


def test_workers_give_the_same_results():
    """Three workers (three engines and host threads) serving a burst: every
    run equals the same run served alone, whichever engine stepped it."""
    eng = api.Engine(api.PREC_MIXED)
    srv = api.Server(eng, max_active=1)
    rid = srv.submit(**_req())
    assert srv.wait(rid)
    alone = srv.result(rid)
    srv.close()

    srv = api.Server(eng, max_active=2, workers=3)
    ids = [srv.submit(**_req()) for _ in range(5)]
    ids += [srv.submit(**_req(eps=-0.3, U=0.6, nsites=10))]
    for i in ids[:5]:
        assert srv.wait(i)
        _same(srv.result(i), alone)
    assert srv.wait(ids[5])
    assert np.isfinite(srv.result(ids[5])["entropy"]).all()
    st = srv.stats()
    srv.close()
    eng.close()
    assert st["completed"] == 6 and st["failed"] == 0
    assert st["max_active_seen"] > 2  # more runs active than one worker may hold


def test_model_mix_alone_and_in_mix_are_equal():
    """A Kondo run (no V site, Lambda 2.5) and a two-channel run (four
    hoppings per site, Lambda 4), each served alone and then in a mix with
    SIAM runs of other Lambda and Nkeep that share its ticks: every site's
    eigenvalues bit for bit."""
    kondo = workloads.flow_request("kondo", 96, 12, 2.5, J=0.2)
    twoch = workloads.flow_request("twochannel", 64, 6, 4.0, V=0.12, eps=-0.3, U=0.6)
    eng = api.Engine(api.PREC_MIXED)
    alone = []
    for req in (kondo, twoch):
        srv = api.Server(eng, max_active=1)
        rid = srv.submit(**req)
        assert srv.wait(rid)
        alone.append(srv.result(rid)["eig"])
        srv.close()
    srv = api.Server(eng, max_active=8)
    ids = [srv.submit(**workloads.flow_request("siam", 128, 10, 3.0, V=0.1, eps=-0.2, U=0.5)),
           srv.submit(**kondo),
           srv.submit(**workloads.flow_request("siam", 64, 14, 2.0, V=0.2, eps=-0.4, U=0.8)),
           srv.submit(**twoch),
           srv.submit(**workloads.flow_request("kondo", 80, 9, 2.5, J=0.08))]
    got = []
    for i in ids:
        assert srv.wait(i)
        got.append(srv.result(i)["eig"])
    st = srv.stats()
    srv.close()
    eng.close()
    assert st["completed"] == 5 and st["failed"] == 0 and st["max_active_seen"] > 1
    for a, b in ((alone[0], got[1]), (alone[1], got[3])):
        assert len(a) == len(b)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
