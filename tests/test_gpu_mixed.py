"""Mixed-precision path (FP32 block solve + FP64-accurate refinement) against
the reference fixtures and the FP64 path, through the C ABI."""
import math

import numpy as np
import pytest

from conftest import golden
from parity import check_eigs, degenerate_weights, eig_tol, max_rel_cv
from nrgplusplus_gb300 import api, workloads
from nrgplusplus_gb300 import models as M
from oracle.nrg_oracle import FdmSpectrumOracle, NrgOracle, broaden

pytestmark = pytest.mark.gpu


def test_mixed_small_against_oracle(mixed_engine):
    imp, bath = M.spinhalf(-0.25, 0.5), M.spinhalf(0, 0)
    run = api.NrgCore(mixed_engine, imp, bath, 128)
    ora = NrgOracle(imp, bath, 128)
    for it in range(-1, 14):
        t = [0.1, 0.1] if it < 0 else [M.hopping(it, 2.0)] * 2
        r = 1.0 if it <= 0 else math.sqrt(2.0)
        run.add_bath_site(t, r)
        ora.add_bath_site(t, r, full_fdag=False)
        for s, h in enumerate(ora.H):
            if h.shape[0] and it < 0:
                U = run.current_hamiltonQ(s)
                assert np.abs(U.T @ U - np.eye(len(U))).max() < 1e-13
        run.update_internal_state()
        ora.update_internal_state()
        assert run.kept_counts == list(ora.kept), it
        assert np.abs(run.all_eigenvalue - ora.all_eigenvalue).max() <= eig_tol(it + 1, 2.0), it
    run.close()


def test_mixed_c1_against_reference(mixed_engine):
    fx = golden("ref_c1_siam_nk512")
    out = workloads.run_nrg(mixed_engine, "siam", 512, 40, 2.0, V=0.1, eps=-0.25, U=0.5)
    check_eigs(fx, out["eig"], 2.0)
    for i in range(40):
        assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    out["run"].close()


def test_mixed_kondo_against_shipped_fixture(mixed_engine):
    fx = golden("shipped_kondo_J0.25")
    out = workloads.run_nrg(mixed_engine, "kondo", 1024, 41, 2.0, J=0.25, thermo=True)
    check_eigs(fx, out["eig"], 2.0)
    assert np.abs(out["entropy"] - fx["entropy"]).max() < 1e-8
    assert max_rel_cv(out["specificHeat"], fx["specificHeat"], fx["temperatureArray"]) < 1e-5
    out["run"].close()


def test_mixed_fdm_spectrum_against_reference(mixed_engine):
    fx = golden("ref_c2_siam_fdm_nk256")
    out = workloads.run_nrg(mixed_engine, "siam", 256, 30, 2.0, V=0.15, eps=-0.4, U=0.8, fdm=True)
    e = FdmSpectrumOracle.energy_points()
    om = np.logspace(-8, 0, 801)
    for ip in range(2):
        for sign, arr in (("Positive", out["GreenFnPositiveWeight"]), ("Negative", out["GreenFnNegativeWeight"])):
            ref = np.zeros(100000)
            ref[fx["GreenFn%sWeight%d_idx" % (sign, ip)]] = fx["GreenFn%sWeight%d_val" % (sign, ip)]
            assert abs(arr[ip].sum() - ref.sum()) < 1e-9
            a = mixed_engine.broaden(e, arr[ip], om, 0.6)
            b = broaden(ref, e, om, 0.6)
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    out["run"].close()


def test_mixed_twochannel_against_reference(mixed_engine):
    fx = golden("ref_twochannel_nk256")
    out = workloads.run_nrg(mixed_engine, "twochannel", 256, 8, 4.0, V=0.12, eps=-0.3, U=0.6)
    check_eigs(fx, out["eig"], 4.0)
    for i in range(8):
        assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    out["run"].close()
