"""Pin the CPU oracle against the reference's own numbers (CPU only).

* shipped_*: datasets the reference ships in examples/entropyKondo/*.h5
* ref_*:     outputs of the reference engine compiled here (oracle/build_ref.sh),
             generated by tests/golden/make_golden.py
"""
import math

import numpy as np
import pytest

from conftest import golden
from parity import check_eigs, degenerate_weights, max_rel_cv, stable_sites
from nrgplusplus_gb300 import models as M
from oracle.nrg_oracle import (FdmSpectrumOracle, NrgOracle, broaden, siam_run,
                               temperature_grid)


def _check_eigs(fx, eigs, lam, offset=0, niter=None):
    return check_eigs(fx, eigs, lam, offset, niter=niter)


CV_RTOL = 1e-5  # specific heat, max relative error over T >= 2.6e-7


@pytest.fixture(scope="module")
def kondo_run():
    return siam_run(M.spinhalf_kondo(0.25, 0.5), M.spinhalf(0, 0), 1024, 41, 2.0, kondo=True,
                    thermo=True, full_fdag=False)


def test_shipped_kondo_eigenvalues(kondo_run):
    fx = golden("shipped_kondo_J0.25")
    _check_eigs(fx, kondo_run["eig"], 2.0)


def test_shipped_kondo_thermodynamics(kondo_run):
    fx = golden("shipped_kondo_J0.25")
    T = temperature_grid()
    assert np.allclose(T, fx["temperatureArray"], rtol=1e-14, atol=0)
    assert np.abs(kondo_run["entropy"] - fx["entropy"]).max() < 1e-8
    # C(T) suffers cancellation at the lowest temperatures (as in the reference itself)
    assert max_rel_cv(kondo_run["cv"], fx["specificHeat"], T) < CV_RTOL


def test_shipped_free_chain_entropy():
    fx = golden("shipped_kondo_zero")
    res = siam_run(M.spinhalf(0, 0), M.spinhalf(0, 0), 1024, 41, 2.0, kondo=True, thermo=True,
                   full_fdag=False)
    _check_eigs(fx, res["eig"], 2.0)
    assert np.abs(res["entropy"] - fx["entropy"]).max() < 1e-8


def test_ref_c1_rgflow():
    fx = golden("ref_c1_siam_nk512")
    res = siam_run(M.spinhalf(-0.25, 0.5), M.spinhalf(0, 0), 512, 40, 2.0, V=0.1, full_fdag=False)
    _check_eigs(fx, res["eig"], 2.0)
    for i in range(40):  # kept-state counts per sector: identical
        assert np.array_equal(np.array(res["kept"][i]), fx["kept%d" % i]), i
        assert np.array_equal(np.array(res["dims"][i]), fx["dims%d" % i]), i
    assert np.allclose(res["eigV"], fx["eig_V"], atol=1e-13)


def test_ref_twochannel_rgflow():
    fx = golden("ref_twochannel_nk256")
    imp = M.duplicate_ops(M.spinhalf(-0.3, 0.6), 2)
    res = siam_run(imp, M.two_channel(), 256, 8, 4.0, V=0.12, full_fdag=False)
    _check_eigs(fx, res["eig"], 4.0)
    for i in range(8):
        assert np.array_equal(np.array(res["kept"][i]), fx["kept%d" % i]), i


def test_ref_twochannel_nk4096_first_sites():
    """The oracle at the two-channel workload's own size (Lambda=4,
    Nkeep=4096): through the first truncation (site 2: 65,792 states in
    blocks up to 4144 rows), every eigenvalue and kept count against the
    reference's run."""
    fx = golden("ref_c3_twochannel_nk4096")
    imp = M.duplicate_ops(M.spinhalf(-0.3, 0.6), 2)
    res = siam_run(imp, M.two_channel(), 4096, 3, 4.0, V=0.12, full_fdag=False)
    _check_eigs(fx, res["eig"], 4.0, niter=3)
    for i in range(3):
        assert np.array_equal(np.array(res["kept"][i]), fx["kept%d" % i]), i


def test_ref_fdag_invariants_and_fdm_small():
    """f-dagger and d-dagger blocks compared through degenerate-subspace sums,
    then the T=0 FDM weights."""
    fx = golden("ref_siam_small_ops")
    imp, bath = M.spinhalf(-0.25, 0.5), M.spinhalf(0, 0)
    res = siam_run(imp, bath, 64, 6, 2.0, V=0.1, track_ops=M.d_dag_chi(), fdm=True, full_fdag=True)
    # re-run with op dumps at each site to compare operator invariants
    n = NrgOracle(imp, bath, 64)
    n.add_bath_site([0.1, 0.1], 1.0)
    n.update_internal_state()
    for it in range(6):
        n.add_bath_site([M.hopping(it, 2.0)] * 2, math.sqrt(2.0) if it else 1.0)
        evq = fx["EQ%d" % it]
        # unpack eigenvalues per sector from the dump
        E, o = [], 0
        while o < evq.size:
            k = int(evq[o])
            E.append(evq[o + 1:o + 1 + k])
            o += 1 + k
        assert len(E) == len(n.eigenvaluesQ)
        for s in range(len(E)):
            assert np.abs(E[s] - n.eigenvaluesQ[s]).max(initial=0) < 1e-12
        for ip in range(2):
            for (i, j), F in n.pre_fdag[ip].items():
                key = "F%d_op%d_%d_%d" % (it, ip, i, j)
                assert key in fx.files, key
                v = fx[key]
                G = v[2:].reshape(int(v[0]), int(v[1]))
                if G.size == 0:
                    continue
                Wa = degenerate_weights(F, n.eigenvaluesQ[i], n.eigenvaluesQ[j], 1e-7)
                Wb = degenerate_weights(G, E[i], E[j], 1e-7)
                assert np.abs(Wa - Wb).max() < 1e-9, key
        n.update_internal_state()
    for ip in range(2):
        for sign, arr in (("Positive", res["pos"]), ("Negative", res["neg"])):
            idx = fx["GreenFn%sWeight%d_idx" % (sign, ip)]
            val = fx["GreenFn%sWeight%d_val" % (sign, ip)]
            ref = np.zeros(arr.shape[1])
            ref[idx] = val
            assert abs(arr[ip].sum() - ref.sum()) < 1e-10
            # bin-wise: identical except weight moved across a bin edge by round-off
            assert np.abs(arr[ip] - ref).sum() < 1e-9 * max(1.0, ref.sum())


def _fdm_ref_arrays(fx, nops=2):
    out = {}
    for sign in ("Positive", "Negative"):
        a = np.zeros((nops, 100000))
        for ip in range(nops):
            a[ip, fx["GreenFn%sWeight%d_idx" % (sign, ip)]] = fx["GreenFn%sWeight%d_val" % (sign, ip)]
        out[sign] = a
    return out


def test_ref_c2_fdm_nk256():
    fx = golden("ref_c2_siam_fdm_nk256")
    res = siam_run(M.spinhalf(-0.4, 0.8), M.spinhalf(0, 0), 256, 30, 2.0, V=0.15,
                   track_ops=M.d_dag_chi(), fdm=True, full_fdag=False)
    _check_eigs(fx, res["eig"], 2.0)
    ref = _fdm_ref_arrays(fx)
    e = FdmSpectrumOracle.energy_points()
    om = np.logspace(-8, 0, 801)
    for ip in range(2):
        for sign, arr in (("Positive", res["pos"]), ("Negative", res["neg"])):
            r = ref[sign][ip]
            assert abs(arr[ip].sum() - r.sum()) < 1e-9
            a = broaden(arr[ip], e, om, 0.6)
            b = broaden(r, e, om, 0.6)
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


def test_ref_kondo_thermo_nk512():
    fx = golden("ref_kondo_thermo_nk512")
    res = siam_run(M.spinhalf_kondo(0.25, 0.5), M.spinhalf(0, 0), 512, 30, 2.0, kondo=True,
                   thermo=True, full_fdag=False)
    _check_eigs(fx, res["eig"], 2.0)
    assert np.abs(res["entropy"] - fx["entropy"]).max() < 1e-8
    assert max_rel_cv(res["cv"], fx["specificHeat"], fx["temperatureArray"]) < CV_RTOL


@pytest.mark.parametrize("k", [2, 3])
def test_ref_sweep_instances(k):
    """Instances of the seeded parameter sweep (Lambda 2.5 and 3) against the
    reference's runs of them."""
    from nrgplusplus_gb300.workloads import sweep_instances
    p = sweep_instances()[k]
    fx = golden("ref_sweep_%03d" % k)
    n = min(p["nsites"], stable_sites(p["lam"]))
    res = siam_run(M.spinhalf(p["eps"], p["U"]), M.spinhalf(0, 0), p["nkeep"], n, p["lam"],
                   V=p["V"], full_fdag=False)
    check_eigs(fx, res["eig"], p["lam"], niter=n)
    for i in range(n):
        assert np.array_equal(np.array(res["kept"][i]), fx["kept%d" % i]), i


def _nd_run(**kw):
    ops = M.d_dag_chi() + M.n_d()
    return siam_run(M.spinhalf(-0.25, 0.8), M.spinhalf(0, 0), 256, 30, 2.0, V=0.15, track_ops=ops,
                    full_fdag=False, **kw)


def test_ref_thermo_system_operator():
    """<n_d>(T) of fdmThermodynamics::setSystemOperator against the reference."""
    fx = golden("ref_siam_thermo_nd_nk256")
    res = _nd_run(thermo=True, sysop_index=[2])
    check_eigs(fx, res["eig"], 2.0)
    assert np.abs(res["entropy"] - fx["entropy"]).max() < 1e-8
    assert np.abs(res["opexp"][0] - fx["qsysOPeratorExpValue0"]).max() < 1e-10


@pytest.mark.parametrize("itemp", [0, 60, 120, 160, 199])
def test_finite_t_static_equals_thermodynamic_average(itemp):
    """Two reference formulas for one number: rhoDotStaticOperators on the
    finite-T FDM density matrix (fdmBackwardIteration.hpp:166-239) and the
    thermodynamic average of the discarded-state diagonals
    (fdmThermodynamics.hpp:63-88, :200-218) give the same <n_d>(T); the
    density matrix has unit trace at every T."""
    T = temperature_grid()[itemp]
    th = _nd_run(thermo=True, sysop_index=[2])
    res = _nd_run(fdm=True, fdm_T=T)
    assert res["static"][0] == 0.0 and res["static"][1] == 0.0  # d-dagger-chi has no (i, i) blocks
    assert abs(res["static"][2] - th["opexp"][0][itemp]) < 1e-12


def test_finite_t_fdm_low_temperature_limit():
    """At the lowest grid temperature the finite-T spectrum is the T = 0 one
    (the ground state lies in the last shell): the same histograms."""
    T = temperature_grid()[0]
    r0 = _nd_run(fdm=True)
    rt = _nd_run(fdm=True, fdm_T=T)
    for a, b in ((r0["pos"], rt["pos"]), (r0["neg"], rt["neg"])):
        assert np.abs(a - b).max() < 1e-12


def test_ref_superconducting_bath():
    """S_z-only sectors and a bath refreshed before every site (the pairing
    grows as Lambda^(n/2) in iteration units) against the reference."""
    fx = golden("ref_sc_nk256")
    delta, lam = 0.001, 2.0
    n = NrgOracle(M.spinhalf_sc(-0.3, 0.6), M.sc_bath(delta), 256)
    n.add_bath_site([0.12, 0.12], 1.0, full_fdag=False)
    n.update_internal_state()
    eigs = []
    for it in range(20):
        n.bath = M.sc_bath(delta * lam ** (0.5 * it))
        n.add_bath_site([M.hopping(it, lam)] * 2, math.sqrt(lam) if it else 1.0, full_fdag=False)
        n.update_internal_state()
        eigs.append(n.all_eigenvalue.copy())
        assert np.array_equal(np.array(n.kept), fx["kept%d" % it]), it
    check_eigs(fx, eigs, lam)
