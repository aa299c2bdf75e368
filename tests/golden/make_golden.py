"""Regenerate the golden fixtures under tests/golden/.

Two sources, both the reference's own numbers:

1. Datasets the reference shipped in examples/entropyKondo/resultsJ0.250000.h5
   and resultsZero.h5 (written by examples/entropyKondo/main.cpp), read with
   the minimal HDF5 walker in h5mini.py.
2. Outputs of the reference engine compiled here by oracle/build_ref.sh
   (oracle/_ref/ref_nrg), for the workloads named in each case below.

Run from the repository root after ``oracle/build_ref.sh``:
    NRG_REF_ROOT=<reference tree> python tests/golden/make_golden.py [names]
The shipped .h5 datasets are read from $NRG_REF_ROOT; the fixtures it writes
are committed so nothing else needs the tree.  Every iteration's eigenvalue
array is stored whole (``eig<i>``), with its count and sum.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from h5mini import H5Mini  # noqa: E402
from oracle.refio import read_named_arrays  # noqa: E402

REF = os.environ.get("NRG_REF_ROOT", "")
BIN = os.path.join(ROOT, "oracle", "_ref", "ref_nrg")


def _eig_entries(out, tag, e):
    out["eig%s" % tag] = e
    out["eig_count%s" % tag] = np.array([e.size])
    out["eig_sum%s" % tag] = np.array([np.sum(e)])


def shipped_h5():
    if not REF:
        raise SystemExit("set NRG_REF_ROOT to the reference tree")
    for tag, fn in (("kondo_J0.25", "resultsJ0.250000.h5"), ("kondo_zero", "resultsZero.h5")):
        h = H5Mini(os.path.join(REF, "examples", "entropyKondo", fn))
        out = {}
        n = 0
        while "Eigenvalues%d" % n in h.datasets:
            _eig_entries(out, n, h.read("Eigenvalues%d" % n))
            n += 1
        out["niter"] = np.array([n])
        for k in ("temperatureArray", "entropy", "specificHeat"):
            out[k] = h.read(k)
        np.savez_compressed(os.path.join(HERE, "shipped_%s.npz" % tag), **out)
        print("shipped", tag, n, "iterations")


def shipped_zaverage():
    """The Wilson-chain coefficients shipped with independFiles/zAverage:
    the flat band at z = 1, Lambda = 3 (hoppingElementsL3.h5, main.cpp) and
    the pseudogap baths |e|^r, r = 1 and 1/2 (pseudoGap3.h5, pseudogap.cpp)."""
    base = os.path.join(REF, "independFiles", "zAverage")
    out = {"flat_tn_z1_L3": H5Mini(os.path.join(base, "hoppingElementsL3.h5")).read("tnZ1.000lmd3.000")}
    h = H5Mini(os.path.join(base, "pseudoGap3.h5"))
    for k in ("tnPseudo", "enPseudo", "tnPseudo2", "enPseudo2"):
        out[k] = h.read(k)
    np.savez_compressed(os.path.join(HERE, "shipped_zaverage.npz"), **out)
    print("shipped zaverage")


def run_ref(model, name, **kw):
    threads = os.environ.get("NRG_REF_THREADS", "8")
    env = dict(os.environ, OMP_NUM_THREADS=threads, OPENBLAS_NUM_THREADS=threads)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "%s.bin" % name)
        args = [BIN, model, path] + ["%s=%r" % (k, v) for k, v in kw.items()]
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, env=env)
        return read_named_arrays(path)


def pack_run(d, with_ops=False, with_fdm=False, with_thermo=False, full_eigs=True):
    out = {}
    iters = sorted(int(k[len("Eigenvalues"):]) for k in d
                   if k.startswith("Eigenvalues") and k[len("Eigenvalues"):].isdigit())
    out["niter"] = np.array([len(iters)])
    for i in iters:
        e = d["Eigenvalues%d" % i]
        _eig_entries(out, i, e if full_eigs else e[:64])
        out["eig_count%d" % i] = np.array([e.size])
        out["eig_sum%d" % i] = np.array([np.sum(e)])
        out["kept%d" % i] = d["kept%d" % i].astype(np.int64)
        out["dims%d" % i] = d["dims%d" % i].astype(np.int64)
    if "EigenvaluesV" in d:
        out["eig_V"] = d["EigenvaluesV"]
    out["relgs"] = d["relativeGroundStateEnergy"]
    out["min_it"] = d["minIterations"]
    if with_ops:
        for k, v in d.items():
            if k.startswith(("F", "D", "EQ")) and "_op" in k or k.startswith("EQ"):
                out[k] = v
    if with_fdm:
        for k, v in d.items():
            if k.startswith("GreenFnPositiveWeight") or k.startswith("GreenFnNegativeWeight"):
                nz = np.nonzero(v)[0]
                out[k + "_idx"] = nz.astype(np.int64)
                out[k + "_val"] = v[nz]
    if with_thermo:
        for k in ("temperatureArray", "entropy", "specificHeat"):
            out[k] = d[k]
        for k, v in d.items():
            if k.startswith("qsysOPeratorExpValue"):
                out[k] = v
    return out


CASES = [
    # (fixture name, model, parameters, what to keep)
    ("ref_c1_siam_nk512", "siam",
     dict(eps=-0.25, U=0.5, V=0.1, **{"lambda": 2.0}, nkeep=512, nsites=40), {}),
    ("ref_siam_small_ops", "siam",
     dict(eps=-0.25, U=0.5, V=0.1, **{"lambda": 2.0}, nkeep=64, nsites=6, fdm=1, dumpops=6),
     {"with_ops": True, "with_fdm": True}),
    ("ref_c2_siam_fdm_nk256", "siam",
     dict(eps=-0.4, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=256, nsites=30, fdm=1),
     {"with_fdm": True}),
    ("ref_c2_siam_fdm_nk1024", "siam",
     dict(eps=-0.4, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=1024, nsites=50, fdm=1),
     {"with_fdm": True}),
    # the same forward run as ref_c2_siam_fdm_nk1024: its eigenvalues are not repeated
    ("ref_c2_siam_thermo_nk1024", "siam",
     dict(eps=-0.4, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=1024, nsites=50, thermo=1),
     {"with_thermo": True, "full_eigs": False}),
    # the spectral workload at Nkeep=2048 (40 Wilson sites)
    ("ref_siam_fdm_nk2048", "siam",
     dict(eps=-0.4, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=2048, nsites=40, fdm=1),
     {"with_fdm": True}),
    ("ref_siam_thermo_nk2048", "siam",
     dict(eps=-0.4, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=2048, nsites=40, thermo=1),
     {"with_thermo": True, "full_eigs": False}),
    ("ref_kondo_thermo_nk512", "kondo",
     dict(J=0.25, **{"lambda": 2.0}, nkeep=512, nsites=30, thermo=1), {"with_thermo": True}),
    # <n_d>(T) through fdmThermodynamics::setSystemOperator (asymmetric SIAM)
    ("ref_siam_thermo_nd_nk256", "siam",
     dict(eps=-0.25, U=0.8, V=0.15, **{"lambda": 2.0}, nkeep=256, nsites=30, thermo=1, sysop=1),
     {"with_thermo": True}),
    # superconducting bath (S_z sectors, pairing refreshed before every site)
    ("ref_sc_nk256", "sc",
     dict(eps=-0.3, U=0.6, V=0.12, **{"lambda": 2.0}, nkeep=256, nsites=20, delta=0.001), {}),
    ("ref_twochannel_nk256", "twochannel",
     dict(eps=-0.3, U=0.6, V=0.12, **{"lambda": 4.0}, nkeep=256, nsites=8), {}),
    # the two-channel workload at its own size (Nkeep=4096, blocks up to ~4300)
    # over its first sites
    ("ref_c3_twochannel_nk4096", "twochannel",
     dict(eps=-0.3, U=0.6, V=0.12, **{"lambda": 4.0}, nkeep=4096, nsites=5), {}),
]


def sweep_cases(count=6):
    """RG flows of the first instances of the seeded SIAM sweep
    (nrgplusplus_gb300.workloads.sweep_instances) with Nkeep <= 1024, each
    Lambda of the sweep represented."""
    from nrgplusplus_gb300.workloads import sweep_instances
    out = []
    for k, p in enumerate(sweep_instances()):
        if p["nkeep"] > 1024:
            continue
        out.append(("ref_sweep_%03d" % k, "siam",
                    dict(eps=p["eps"], U=p["U"], V=p["V"], **{"lambda": p["lam"]}, nkeep=p["nkeep"],
                         nsites=p["nsites"]), {}))
        if len(out) == count:
            break
    return out


def main(which=None):
    if not which:
        shipped_h5()
        shipped_zaverage()
    for name, model, params, opts in CASES + sweep_cases():
        if which and name not in which:
            continue
        d = run_ref(model, name, **params)
        out = pack_run(d, **opts)
        out["params"] = np.array([repr((model, params))])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
