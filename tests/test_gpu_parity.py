"""GPU engine vs the CPU oracle and the reference's golden fixtures, through
the C ABI (FP64 path).  Tolerances: tests/parity.py."""
import math

import numpy as np
import pytest

from conftest import golden
from parity import check_eigs, degenerate_weights, eig_tol, max_rel_cv
from nrgplusplus_gb300 import api, workloads
from nrgplusplus_gb300 import models as M
from oracle.nrg_oracle import FdmSpectrumOracle, NrgOracle, broaden, siam_run

pytestmark = pytest.mark.gpu


def _eigs_match(gpu, ref, lam, offset=0):
    assert len(gpu) == len(ref)
    for i, (a, b) in enumerate(zip(gpu, ref)):
        assert a.shape == b.shape, i
        assert np.abs(a - b).max() <= eig_tol(i + offset, lam), (i, np.abs(a - b).max())


def test_small_siam_step_by_step(gpu_engine):
    """Every public member after every step, against the oracle."""
    imp, bath = M.spinhalf(-0.25, 0.5), M.spinhalf(0, 0)
    run = api.NrgCore(gpu_engine, imp, bath, 64)
    ora = NrgOracle(imp, bath, 64)
    for it in range(-1, 10):
        t = [0.1, 0.1] if it < 0 else [M.hopping(it, 2.0)] * 2
        r = 1.0 if it <= 0 else math.sqrt(2.0)
        run.add_bath_site(t, r)
        ora.add_bath_site(t, r, full_fdag=True)
        # between add_bath_site and update_internal_state
        assert run.current_sysmQ == [tuple(q) for q in ora.current_sysmQ]
        assert run.coupled_nQ_index == ora.coupled
        ev = run.eigenvaluesQ
        assert len(ev) == len(ora.eigenvaluesQ)
        for a, b in zip(ev, ora.eigenvaluesQ):
            assert a.shape == b.shape
            assert np.abs(a - b).max(initial=0) < 1e-11
        kept_next = [int(np.count_nonzero(e < np.sort(np.concatenate(ora.eigenvaluesQ))[64] + 1e-8))
                     if sum(len(x) for x in ora.eigenvaluesQ) > 64 else len(e) for e in ora.eigenvaluesQ]
        for ip in range(2):
            for (i, j), F in ora.pre_fdag[ip].items():
                G = run.fdag_block(ip, i, j)
                ki, kj = kept_next[i], kept_next[j]
                if ki == 0 or kj == 0:
                    assert G is None
                    continue
                assert G is not None and G.shape == (ki, kj), (ip, i, j)
                Wa = degenerate_weights(F[:ki, :kj], ora.eigenvaluesQ[i][:ki], ora.eigenvaluesQ[j][:kj], 1e-7)
                Wb = degenerate_weights(G, ev[i][:ki], ev[j][:kj], 1e-7)
                assert np.abs(Wa - Wb).max() < 1e-9, (it, ip, i, j)
        # eigenvectors: orthonormal columns; at the first site both engines
        # assemble H from the same impurity operators, so U must diagonalise
        # the oracle's H (later sites differ by the arbitrary sign gauge of
        # the previous eigenvectors)
        for s, h in enumerate(ora.H):
            if h.shape[0]:
                U = run.current_hamiltonQ(s)
                assert np.abs(U.T @ U - np.eye(len(U))).max() < 1e-12
                if it < 0:
                    assert np.abs(U.T @ h @ U - np.diag(ev[s])).max() < 1e-11
        run.update_internal_state()
        ora.update_internal_state()
        assert np.abs(run.all_eigenvalue - ora.all_eigenvalue).max() < 1e-11
        assert run.kept_counts == list(ora.kept)
        assert run.pre_sysmQ == [tuple(q) for q in ora.pre_sysmQ]
        assert run.nrg_iterations_cnt == ora.nrg_iterations_cnt
        assert run.nrg_iterations_min == ora.nrg_iterations_min
        assert np.allclose(run.relativeGroundStateEnergy, ora.relativeGroundStateEnergy, atol=1e-12)
        assert run.checkHigherEnergyDiscarded() == ora.checkHigherEnergyDiscarded()
        for a, b in zip(run.eigenvaluesQ, ora.eigenvaluesQ):
            assert np.abs(a - b).max(initial=0) < 1e-11
    run.close()


def test_c1_rgflow_against_reference(gpu_engine):
    fx = golden("ref_c1_siam_nk512")
    out = workloads.run_nrg(gpu_engine, "siam", 512, 40, 2.0, V=0.1, eps=-0.25, U=0.5)
    check_eigs(fx, out["eig"], 2.0)
    for i in range(40):
        assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    out["run"].close()


def test_kondo_against_shipped_fixture(gpu_engine):
    fx = golden("shipped_kondo_J0.25")
    out = workloads.run_nrg(gpu_engine, "kondo", 1024, 41, 2.0, J=0.25, thermo=True)
    check_eigs(fx, out["eig"], 2.0)
    assert np.abs(out["entropy"] - fx["entropy"]).max() < 1e-8
    assert max_rel_cv(out["specificHeat"], fx["specificHeat"], fx["temperatureArray"]) < 1e-5
    out["run"].close()


def test_twochannel_against_reference(gpu_engine):
    fx = golden("ref_twochannel_nk256")
    out = workloads.run_nrg(gpu_engine, "twochannel", 256, 8, 4.0, V=0.12, eps=-0.3, U=0.6)
    check_eigs(fx, out["eig"], 4.0)
    for i in range(8):
        assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    out["run"].close()


def test_fdm_spectrum_against_reference(gpu_engine):
    fx = golden("ref_c2_siam_fdm_nk256")
    out = workloads.run_nrg(gpu_engine, "siam", 256, 30, 2.0, V=0.15, eps=-0.4, U=0.8, fdm=True)
    e = FdmSpectrumOracle.energy_points()
    assert np.allclose(out["GreenFnEnergyPoints"], e, rtol=1e-15)
    om = np.logspace(-8, 0, 801)
    for ip in range(2):
        for sign, arr in (("Positive", out["GreenFnPositiveWeight"]), ("Negative", out["GreenFnNegativeWeight"])):
            ref = np.zeros(100000)
            ref[fx["GreenFn%sWeight%d_idx" % (sign, ip)]] = fx["GreenFn%sWeight%d_val" % (sign, ip)]
            assert abs(arr[ip].sum() - ref.sum()) < 1e-9
            a = gpu_engine.broaden(e, arr[ip], om, 0.6)
            b = broaden(ref, e, om, 0.6)
            assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    out["run"].close()


def test_tracked_operator_invariants(gpu_engine):
    imp, bath = M.spinhalf(-0.4, 0.8), M.spinhalf(0, 0)
    run = api.NrgCore(gpu_engine, imp, bath, 96)
    ora = NrgOracle(imp, bath, 96)
    ops = api.OperatorSet(run, M.d_dag_chi())
    oops = M.d_dag_chi()
    for it in range(-1, 8):
        t = [0.15, 0.15] if it < 0 else [M.hopping(it, 2.0)] * 2
        r = 1.0 if it <= 0 else math.sqrt(2.0)
        run.add_bath_site(t, r)
        ora.add_bath_site(t, r, full_fdag=False)
        api.update_system_operator(run, ops)
        oops = ora.update_system_operator(oops)
        ev = ora.eigenvaluesQ
        for ip in range(2):
            for (i, j), O in oops[ip].items():
                G = ops.block(ip, i, j)
                if O.size == 0:
                    continue
                if G is None:  # the engine omits blocks built only from empty sub-blocks
                    assert np.abs(O).max() == 0.0, (it, ip, i, j)
                    continue
                assert G.shape == O.shape
                Wa = degenerate_weights(O, ev[i], ev[j], 1e-7)
                Wb = degenerate_weights(G, ev[i], ev[j], 1e-7)
                assert np.abs(Wa - Wb).max() < 1e-9, (it, ip, i, j)
        run.update_internal_state()
        ora.update_internal_state()
    run.close()


def test_batched_runs_equal_single_runs(gpu_engine):
    params = [(-0.25, 0.5, 0.1, 128), (-0.4, 0.8, 0.15, 96), (-0.1, 0.3, 0.2, 160)]
    singles = []
    for eps, U, V, nk in params:
        o = workloads.run_nrg(gpu_engine, "siam", nk, 12, 2.0, V=V, eps=eps, U=U)
        singles.append(o["eig"])
        o["run"].close()
    runs = [api.NrgCore(gpu_engine, M.spinhalf(eps, U), M.spinhalf(0, 0), nk) for eps, U, V, nk in params]
    api.batch_add_site(runs, [[V, V] for _, _, V, _ in params], [1.0] * 3)
    api.batch_update_state(runs)
    for it in range(12):
        api.batch_add_site(runs, [[M.hopping(it, 2.0)] * 2] * 3, [math.sqrt(2.0) if it else 1.0] * 3)
        api.batch_update_state(runs)
        for k, r in enumerate(runs):
            assert np.array_equal(r.all_eigenvalue, singles[k][it]), (it, k)  # bit-identical
    for r in runs:
        r.close()


def test_errors_are_reported(gpu_engine):
    run = api.NrgCore(gpu_engine, M.spinhalf(-0.25, 0.5), M.spinhalf(0, 0), 32)
    with pytest.raises(api.NrgError):
        run.add_bath_site([0.1, 0.1, 0.1], 1.0)  # hopping count (nrgcore.hpp:148-152)
    run.add_bath_site([0.1, 0.1], 1.0)
    with pytest.raises(api.NrgError):
        run.add_bath_site([0.1, 0.1], 1.0)  # add twice without update
    run.update_internal_state()
    with pytest.raises(api.NrgError):
        run.update_internal_state()  # update twice
    run.close()
