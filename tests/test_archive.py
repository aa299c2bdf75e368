"""The snapshot export container (nrgplusplus_gb300.archive): the format
round trip on the CPU, and on the GPU an exported run against the oracle's
in-memory snapshots of the same run (NrgData's members, nrgData.hpp:134-293)."""
import math

import numpy as np
import pytest

from parity import degenerate_weights
from nrgplusplus_gb300 import archive


def test_container_round_trip(tmp_path):
    arrays = {"/NrgItr3/eigenvaluesQ/0": np.array([0.0, 1.5, 2.25]), "empty": np.zeros(0),
              "Eigenvalues7": np.linspace(-1, 1, 5)}
    p = str(tmp_path / "a.bin")
    archive.write(p, arrays)
    back = archive.read(p)
    assert list(back) == list(arrays)
    for k in arrays:
        assert np.array_equal(back[k], arrays[k])
    with open(p, "r+b") as f:
        f.write(b"XXXX")
    with pytest.raises(ValueError):
        archive.read(p)


@pytest.mark.gpu
def test_export_matches_oracle_snapshots(gpu_engine, tmp_path):
    from nrgplusplus_gb300 import api
    from nrgplusplus_gb300 import models as M
    from oracle.nrg_oracle import siam_run
    imp, bath = M.spinhalf(-0.4, 0.8), M.spinhalf(0, 0)
    nk, ns = 128, 10
    run = api.NrgCore(gpu_engine, imp, bath, nk)
    data = api.NrgData(run)
    ops = api.OperatorSet(run, M.d_dag_chi())
    run.add_bath_site([0.15, 0.15], 1.0)
    api.update_system_operator(run, ops)
    run.update_internal_state()
    for it in range(ns):
        run.add_bath_site([M.hopping(it, 2.0)] * 2, math.sqrt(2.0) if it else 1.0)
        api.update_system_operator(run, ops)
        if run.checkHigherEnergyDiscarded():
            data.saveCurrentData(ops)
        run.update_internal_state()
    path = str(tmp_path / "snap.bin")
    data.export(path)
    got = archive.read(path)
    ref = siam_run(imp, bath, nk, ns, 2.0, V=0.15, track_ops=M.d_dag_chi(), fdm=True, full_fdag=False)
    saved = got["savedNRGIndex"].astype(int).tolist()
    assert saved == sorted(ref["snaps"])
    assert np.allclose(got["relativeGroundStateEnergy"], run.relativeGroundStateEnergy, atol=0)
    for it in saved:
        sh = archive.shell(got, it)
        rs = ref["snaps"][it]
        assert sh["current_sysmQ"] == [tuple(q) for q in rs["current_sysmQ"]]
        assert sh["pre_sysmQ"] == [tuple(q) for q in rs["pre_sysmQ"]]
        assert sh["eigenvaluesQ_kept_indices"] == list(rs["kept"])
        assert sh["coupled_nQ_index"] == [list(c) for c in rs["coupled"]]
        for a, b in zip(sh["eigenvaluesQ"], rs["eigenvaluesQ"]):
            assert a.shape == b.shape and np.abs(a - b).max(initial=0) < 1e-10
        for U in sh["current_hamiltonQ"]:
            if U.size:
                assert np.abs(U.T @ U - np.eye(len(U))).max() < 1e-12
        for ip in range(2):
            for (i, j), O in rs["ops"][ip].items():
                G = sh["ops"][ip].get((i, j))
                if O.size == 0 or G is None:
                    continue
                Wa = degenerate_weights(O, rs["eigenvaluesQ"][i], rs["eigenvaluesQ"][j], 1e-7)
                Wb = degenerate_weights(G, sh["eigenvaluesQ"][i], sh["eigenvaluesQ"][j], 1e-7)
                assert np.abs(Wa - Wb).max() < 1e-9, (it, ip, i, j)
    run.close()
