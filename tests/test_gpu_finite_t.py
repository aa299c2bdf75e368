"""Finite-temperature FDM and the system-operator averages on the GPU, both
precision paths, through the C ABI.

* <n_d>(T) of the thermodynamics (fdmThermodynamics::setSystemOperator)
  against the reference's own output (tests/golden/ref_siam_thermo_nd_nk256).
* The FDM spectrum at temperature T (each shell's discarded states carry the
  thermodynamic Boltzmann weights, the fdmBackwardIteration::setRhoZero(
  tBoltzmannFactor) form) and the static <n_d>(T) of rhoDotStaticOperators
  against the CPU oracle on the same run; the oracle's finite-T density
  matrix is pinned by tests/test_oracle_golden.py (its static <n_d>(T)
  equals the reference's thermodynamic average, its T -> 0 limit the
  reference's T = 0 spectrum)."""
import numpy as np
import pytest

from conftest import golden
from parity import check_eigs
from nrgplusplus_gb300 import models as M
from nrgplusplus_gb300 import workloads
from oracle.nrg_oracle import FdmSpectrumOracle, broaden, siam_run, temperature_grid

pytestmark = pytest.mark.gpu

PARAMS = dict(V=0.15, eps=-0.25, U=0.8)


@pytest.mark.parametrize("path", ["fp64", "mixed"])
def test_thermo_system_operator_against_reference(gpu_engine, mixed_engine, path):
    eng = gpu_engine if path == "fp64" else mixed_engine
    fx = golden("ref_siam_thermo_nd_nk256")
    out = workloads.run_nrg(eng, "siam", 256, 30, 2.0, thermo=True, with_nd=True, **PARAMS)
    try:
        check_eigs(fx, out["eig"], 2.0)
        assert np.abs(out["entropy"] - fx["entropy"]).max() < 1e-8
        assert np.abs(out["qsysOPeratorExpValue"][0] - fx["qsysOPeratorExpValue0"]).max() < 1e-9
    finally:
        out["run"].close()


@pytest.mark.parametrize("path", ["fp64", "mixed"])
@pytest.mark.parametrize("itemp", [100, 150])
def test_finite_t_fdm_against_oracle(gpu_engine, mixed_engine, path, itemp):
    eng = gpu_engine if path == "fp64" else mixed_engine
    T = float(temperature_grid()[itemp])
    out = workloads.run_nrg(eng, "siam", 256, 30, 2.0, fdm=True, fdm_T=T, with_nd=True, **PARAMS)
    ref = siam_run(M.spinhalf(PARAMS["eps"], PARAMS["U"]), M.spinhalf(0, 0), 256, 30, 2.0, V=PARAMS["V"],
                   track_ops=M.d_dag_chi() + M.n_d(), fdm=True, fdm_T=T, full_fdag=False)
    try:
        assert np.abs(out["static"] - ref["static"]).max() < 1e-9
        e = FdmSpectrumOracle.energy_points()
        om = np.logspace(-8, 0, 801)
        for ip in range(2):
            for a, b in ((out["GreenFnPositiveWeight"][ip], ref["pos"][ip]),
                         (out["GreenFnNegativeWeight"][ip], ref["neg"][ip])):
                assert abs(a.sum() - b.sum()) < 1e-9
                ga = eng.broaden(e, a, om, 0.6)
                gb = broaden(b, e, om, 0.6)
                assert np.abs(ga - gb).max() <= 1e-6 * np.abs(gb).max()
    finally:
        out["run"].close()
