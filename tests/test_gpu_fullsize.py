"""Parity at the benchmarked sizes, both precision paths, through the C ABI:

* the spectral workload (eps_d=-0.4, U=0.8, V=0.15, Lambda=2) at Nkeep=1024 /
  50 sites and at Nkeep=2048 / 40 sites, d-dagger-chi tracked, T=0 FDM
  spectrum, entropy and specific heat, against the reference's own outputs
  (tests/golden/ref_c2_siam_*_nk1024, ref_siam_*_nk2048);
* the two-channel workload at its own size (Lambda=4, Nkeep=4096, blocks up
  to 4279 rows), both paths, over its first five sites, against the
  reference's run (tests/golden/ref_c3_twochannel_nk4096);
* instances of the seeded parameter sweep stepped together in one batch
  (different Lambda, Nkeep and lengths), against the reference's outputs for
  each instance (tests/golden/ref_sweep_*), over the sites where the
  reference's own FP64 noise stays below the truncation window
  (tests/parity.py: stable_sites).

Every eigenvalue of every iteration is compared (tests/parity.py:
check_eigs), kept counts per block exactly, the FDM histograms through their
sums (1e-9) and the broadened spectral function (1e-6 of its maximum), the
entropy to 1e-8 and the specific heat by its largest relative error over
T >= 2.6e-7."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
from parity import check_eigs, max_rel_cv, stable_sites
from nrgplusplus_gb300 import workloads
from oracle.nrg_oracle import FdmSpectrumOracle, broaden

pytestmark = pytest.mark.gpu

CV_RTOL = 1e-5
SPEC_RTOL = 1e-6


def _spectral_run(engine, nkeep, nsites):
    return workloads.run_nrg(engine, "siam", nkeep, nsites, 2.0, V=0.15, eps=-0.4, U=0.8, fdm=True,
                             thermo=True)


def _check_spectral(engine, out, fdm_fx, thermo_fx, nsites):
    check_eigs(fdm_fx, out["eig"], 2.0)
    for i in range(nsites):
        assert np.array_equal(np.array(out["kept"][i]), fdm_fx["kept%d" % i]), i
    e = FdmSpectrumOracle.energy_points()
    om = np.logspace(-8, 0, 801)
    for ip in range(2):
        for sign, arr in (("Positive", out["GreenFnPositiveWeight"]),
                          ("Negative", out["GreenFnNegativeWeight"])):
            ref = np.zeros(100000)
            ref[fdm_fx["GreenFn%sWeight%d_idx" % (sign, ip)]] = fdm_fx["GreenFn%sWeight%d_val" % (sign, ip)]
            assert abs(arr[ip].sum() - ref.sum()) < 1e-9
            a = engine.broaden(e, arr[ip], om, 0.6)
            b = broaden(ref, e, om, 0.6)
            assert np.abs(a - b).max() <= SPEC_RTOL * np.abs(b).max()
    assert np.abs(out["entropy"] - thermo_fx["entropy"]).max() < 1e-8
    assert max_rel_cv(out["specificHeat"], thermo_fx["specificHeat"], thermo_fx["temperatureArray"]) < CV_RTOL


@pytest.mark.parametrize("path", ["fp64", "mixed"])
def test_spectral_workload_nk1024(gpu_engine, mixed_engine, path):
    eng = gpu_engine if path == "fp64" else mixed_engine
    out = _spectral_run(eng, 1024, 50)
    try:
        _check_spectral(eng, out, golden("ref_c2_siam_fdm_nk1024"), golden("ref_c2_siam_thermo_nk1024"), 50)
    finally:
        out["run"].close()


@pytest.mark.parametrize("path", ["fp64", "mixed"])
def test_spectral_workload_nk2048(gpu_engine, mixed_engine, path):
    eng = gpu_engine if path == "fp64" else mixed_engine
    out = _spectral_run(eng, 2048, 40)
    try:
        _check_spectral(eng, out, golden("ref_siam_fdm_nk2048"), golden("ref_siam_thermo_nk2048"), 40)
    finally:
        out["run"].close()


def _sweep_fixtures():
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "ref_sweep_*.npz")))
    return [(int(n.split("_")[-1]), golden(n)) for n in names]


@pytest.mark.parametrize("path", ["fp64", "mixed"])
def test_sweep_instances_batched(gpu_engine, mixed_engine, path):
    """Heterogeneous batch: the fixture instances of the seeded sweep run as
    one batch; each must equal the reference's run of that instance alone."""
    eng = gpu_engine if path == "fp64" else mixed_engine
    fx = _sweep_fixtures()
    assert len(fx) >= 4
    inst = workloads.sweep_instances()
    params = [inst[k] for k, _ in fx]
    assert len({p["lam"] for p in params}) >= 2
    outs = workloads.run_flow_batch(eng, params)
    for (k, f), p, o in zip(fx, params, outs):
        assert len(o["eig"]) == p["nsites"]
        n = min(p["nsites"], stable_sites(p["lam"]))
        check_eigs(f, o["eig"], p["lam"], niter=n)
        for i in range(n):
            assert np.array_equal(np.array(o["kept"][i]), f["kept%d" % i]), (k, i)


@pytest.mark.parametrize("path", ["fp64", "mixed"])
def test_superconducting_bath_against_reference(gpu_engine, mixed_engine, path):
    """S_z-only sectors (one quantum number) and a pairing bath refreshed
    before every site (set_bath), against the reference's run."""
    eng = gpu_engine if path == "fp64" else mixed_engine
    fx = golden("ref_sc_nk256")
    out = workloads.run_sc(eng, 256, 20, 2.0, V=0.12, eps=-0.3, U=0.6, delta=0.001)
    try:
        check_eigs(fx, out["eig"], 2.0)
        for i in range(20):
            assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    finally:
        out["run"].close()


@pytest.mark.parametrize("path", ["mixed", "fp64"])
def test_two_channel_workload_nk4096(gpu_engine, mixed_engine, path):
    """Blocks of up to 4279 rows (four per site above 4100).  Mixed path: the
    FP32 reflector solver streaming them from global memory, then the
    FP64-accurate refinement; a few blocks miss its convergence test and are
    re-solved in FP64 (the engine's fallback, counted by fallback_count).
    Plain FP64 path: every block above shared memory by the FP64 reflector
    solver (4-column back-transform tiles for the largest)."""
    eng = gpu_engine if path == "fp64" else mixed_engine
    fx = golden("ref_c3_twochannel_nk4096")
    out = workloads.run_nrg(eng, "twochannel", 4096, 5, 4.0, V=0.12, eps=-0.3, U=0.6)
    try:
        check_eigs(fx, out["eig"], 4.0)
        for i in range(5):
            assert np.array_equal(np.array(out["kept"][i]), fx["kept%d" % i]), i
    finally:
        out["run"].close()
