"""Batched calls across runs give the per-run results: nrg_opset_update_batch
bit for bit (fixed-order GEMMs), nrg_fdm_calc_batch to 1e-12 relative (the
binning adds with floating-point atomics)."""
import math

import numpy as np
import pytest

from nrgplusplus_gb300 import api, workloads
from nrgplusplus_gb300 import models as M

pytestmark = pytest.mark.gpu

NK, NS, LAM = 96, 14, 2.0
PARAMS = [(-0.4, 0.8, 0.15), (-0.3, 0.6, 0.12), (-0.5, 1.0, 0.2)]


def _forward(engine, batched_ops=False):
    runs, datas, ops, min_it = [], [], [], []
    for eps, U, V in PARAMS:
        imp, bath = workloads.build_models("siam", eps, U)
        runs.append(api.NrgCore(engine, imp, bath, NK))
        datas.append(api.NrgData(runs[-1]))
    api.batch_add_site(runs, [[V, V] for _, _, V in PARAMS], [1.0] * len(runs))
    ops = [api.OperatorSet(r, M.d_dag_chi()) for r in runs]
    for r, o in zip(runs, ops):
        api.update_system_operator(r, o)
    api.batch_update_state(runs)
    min_it = [0] * len(runs)
    for it in range(NS):
        h = M.hopping(it, LAM)
        api.batch_add_site(runs, [[h, h]] * len(runs), [math.sqrt(LAM) if it > 0 else 1.0] * len(runs))
        if batched_ops:
            api.update_system_operator_batch(runs, ops)
        else:
            for k, r in enumerate(runs):
                api.update_system_operator(r, ops[k])
        for k, r in enumerate(runs):
            if r.checkHigherEnergyDiscarded():
                datas[k].saveCurrentData(ops[k])
            else:
                min_it[k] += 1
        api.batch_update_state(runs)
    return runs, datas, ops, min_it


def _backward(engine, batched):
    runs, datas, ops, min_it = _forward(engine)
    fs = [api.FdmSpectrum(r, 2) for r in runs]
    cnt = [r.nrg_iterations_cnt for r in runs]
    for it in range(NS, min(min_it), -1):
        todo = [k for k in range(len(runs)) if it > min_it[k]]
        for k in todo:
            cnt[k] -= 1
            datas[k].loadCurrentData(cnt[k])
        sc = LAM ** (-(it - 1.0) / 2.0)
        if batched:
            api.fdm_calc_batch([fs[k] for k in todo], [sc] * len(todo))
        else:
            for k in todo:
                fs[k].calcSpectrum(sc)
    out = [f.saveFinalData() for f in fs]
    for f, o, r in zip(fs, ops, runs):
        f.close()
        o.close()
        r.close()
    return out


def test_batched_fdm_equals_per_run(mixed_engine):
    one = _backward(mixed_engine, False)
    many = _backward(mixed_engine, True)
    for a, b in zip(one, many):
        for k in ("GreenFnPositiveWeight", "GreenFnNegativeWeight"):
            assert np.abs(a[k]).sum() > 0
            assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-300)


def test_batched_fdm_rejects_two_objects_of_one_run(mixed_engine):
    imp, bath = workloads.build_models("siam", -0.4, 0.8)
    run = api.NrgCore(mixed_engine, imp, bath, 32)
    run.add_bath_site([0.1, 0.1], 1.0)
    run.update_internal_state()
    f1, f2 = api.FdmSpectrum(run, 2), api.FdmSpectrum(run, 2)
    with pytest.raises(api.NrgError):
        api.fdm_calc_batch([f1, f2], [1.0, 1.0])
    f1.close()
    f2.close()
    run.close()


def test_batched_operator_update_equals_per_run(mixed_engine):
    res = []
    for batched in (False, True):
        runs, datas, ops, _ = _forward(mixed_engine, batched_ops=batched)
        nsec = len(runs[0].eigenvaluesQ)
        blocks = {}
        for k, o in enumerate(ops):
            for ip in range(2):
                for i in range(nsec):
                    for j in range(nsec):
                        b = o.block(ip, i, j)
                        if b is not None:
                            blocks[(k, ip, i, j)] = b
        res.append(blocks)
        for o, r in zip(ops, runs):
            o.close()
            r.close()
    assert res[0].keys() == res[1].keys() and len(res[0]) > 0
    for key in res[0]:
        assert np.array_equal(res[0][key], res[1][key]), key
