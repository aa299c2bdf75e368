"""Workload drivers: the reference's example mains re-expressed over the GPU
API (forward RG flow, operator tracking, FDM backward pass, thermodynamics).

  SIAM RG flow        examples/rgflowSIAM/main.cpp:11-46
  Kondo               examples/rgflowKondo/main.cpp:12-43, entropyKondo/main.cpp:35-119
  two-channel SIAM    examples/twoChannelSiam/main.cpp:13-66
  FDM spectrum        examples/fdmSpectrumSiam/main.cpp:15-141 (2 hoppings for
                      the single-channel spinhalf bath, as rgflowSIAM uses)
  thermodynamics      examples/entropySIAM/main.cpp:13-97
"""
import math

import numpy as np

from . import api
from . import models as M


def temperature_grid(points=200, tmin=1e-10, tmax=2.0):
    """examples/entropySIAM/main.cpp:68-76."""
    d = (points - 1.0) / math.log(tmax / tmin)
    return tmin * np.exp(np.arange(points) / d)


def build_models(kind, eps=-0.25, U=0.5, J=0.25):
    if kind == "siam":
        return M.spinhalf(eps, U), M.spinhalf(0.0, 0.0)
    if kind == "kondo":
        return M.spinhalf_kondo(J, 0.5), M.spinhalf(0.0, 0.0)
    if kind == "zero":
        return M.spinhalf(0.0, 0.0), M.spinhalf(0.0, 0.0)
    if kind == "twochannel":
        return M.duplicate_ops(M.spinhalf(eps, U), 2), M.two_channel()
    raise ValueError(kind)


def run_nrg(engine, kind, nkeep, nsites, lam, V=None, eps=-0.25, U=0.5, J=0.25, fdm=False,
            thermo=False, keep_eigs=True, fdm_T=None, with_nd=False):
    """One NRG run through the public API.  Kondo-type impurities ('kondo',
    'zero') have no V site and rescale by sqrt(Lambda) from the first site.
    fdm_T: the FDM spectrum at that temperature (a thermodynamics pass over
    the same shells first provides the Boltzmann weights) instead of T = 0.
    with_nd: n_d is tracked beside d-dagger-chi (operator 2) and averaged by
    the thermodynamics (qsysOPeratorExpValue) and the FDM (static)."""
    imp, bath = build_models(kind, eps, U, J)
    kondo = kind in ("kondo", "zero")
    nops = len(imp.fdag)
    run = api.NrgCore(engine, imp, bath, nkeep)
    data = api.NrgData(run)
    track = M.d_dag_chi() + (M.n_d() if with_nd else [])
    ops = None
    out = {"eig": [], "kept": [], "run": run}
    if not kondo:
        run.add_bath_site([V] * nops, 1.0)
        if fdm or with_nd:
            ops = api.OperatorSet(run, track)
            api.update_system_operator(run, ops)
        run.update_internal_state()
    min_it = 0
    for it in range(nsites):
        r = math.sqrt(lam) if (kondo or it > 0) else 1.0
        run.add_bath_site([M.hopping(it, lam)] * nops, r)
        if fdm or with_nd:
            if ops is None:
                ops = api.OperatorSet(run, track)
            api.update_system_operator(run, ops)
        if fdm or thermo:
            if run.checkHigherEnergyDiscarded():
                data.saveCurrentData(ops)
            else:
                min_it += 1
        run.update_internal_state()
        if keep_eigs:
            out["eig"].append(run.all_eigenvalue)
            out["kept"].append(run.kept_counts)
    out["min_it"] = min_it
    out["nsites"] = nsites
    last = run.nrg_iterations_cnt  # loadCurrentData moves the counter (nrgData.hpp:273)

    def thermo_pass(temps):
        th = api.FdmThermodynamics(run, temps)
        if with_nd:
            th.setSystemOperator([2])
        cnt = last
        lo = min_it + (1 if kondo else 0)
        for it in range(nsites, lo, -1):
            cnt -= 1
            data.loadCurrentData(cnt)
            th.calcThermodynamics(lam ** (-(1.0 * it - 1.0) / 2.0))
        return th

    if fdm:
        tw = None
        if fdm_T is not None:
            if kondo:
                raise ValueError("finite-T FDM: the thermodynamic shells of a Kondo run start one later")
            tw = thermo_pass([fdm_T])
        f = api.FdmSpectrum(run, ops.nops)
        if tw is not None:
            f.setTemperature(fdm_T, tw)
        cnt = last
        for it in range(nsites, min_it, -1):
            cnt -= 1
            data.loadCurrentData(cnt)
            f.calcSpectrum(lam ** (-(it - 1.0) / 2.0))
        out.update(f.saveFinalData())
        out["static"] = f.staticExpectation()
        f.close()
        if tw is not None:
            tw.close()
    if thermo:
        th = thermo_pass(temperature_grid())
        out.update(th.saveFinalData())
        th.close()
    return out


def spectral_function(engine, energies, pos, neg, b=0.6, decades=(-8, 0), per_decade=100):
    """Log-Gaussian broadened A(w) on 100 points per decade over |w| in
    [1e-8, 1] (spec.py:27-44 form, without the pi*Gamma display factor)."""
    n = (decades[1] - decades[0]) * per_decade + 1
    om = np.logspace(decades[0], decades[1], n)
    return om, engine.broaden(energies, pos, om, b), engine.broaden(energies, neg, om, b)


def siam_request(nkeep, nsites, lam, V, eps=-0.25, U=0.5, fdm=False, thermo=False, keep_eigs=True):
    """Keyword arguments of Server.submit for the SIAM run that run_nrg(...,
    'siam', ...) drives through the API: the V site, then nsites Wilson sites;
    shells kept after the Wilson sites, scaled Lambda^(-(it-1)/2) as in the
    backward loops of run_nrg (examples/fdmSpectrumSiam, examples/entropySIAM)."""
    imp, bath = build_models("siam", eps, U)
    nops = len(imp.fdag)
    t = [[V] * nops] + [[M.hopping(it, lam)] * nops for it in range(nsites)]
    rescale = [1.0] + [math.sqrt(lam) if it > 0 else 1.0 for it in range(nsites)]
    scale = [1.0] + [lam ** (-(it) / 2.0) for it in range(nsites)]
    return dict(impurity=imp, bath=bath, nkeep=nkeep, t=np.array(t), rescale=np.array(rescale),
                ops=M.d_dag_chi() if fdm else None, fdm=fdm,
                temps=temperature_grid() if thermo else None, shell_scale=np.array(scale),
                first_shell_site=1, keep_eigenvalues=keep_eigs)


def run_sc(engine, nkeep, nsites, lam, V, eps, U, delta, keep_eigs=True):
    """SIAM coupled to a superconducting bath: S_z-only sectors
    (models.spinhalf_sc) and a pairing delta Lambda^(n/2) on Wilson site n
    (delta on the V site), the bath refreshed before every site through
    set_bath, as nrgcore re-reads its bath model (nrgcore.hpp:68-70)."""
    run = api.NrgCore(engine, M.spinhalf_sc(eps, U), M.sc_bath(delta), nkeep)
    out = {"eig": [], "kept": [], "run": run}
    run.add_bath_site([V, V], 1.0)
    run.update_internal_state()
    for it in range(nsites):
        run.set_bath(M.sc_bath(delta * lam ** (0.5 * it)))
        run.add_bath_site([M.hopping(it, lam)] * 2, math.sqrt(lam) if it > 0 else 1.0)
        run.update_internal_state()
        if keep_eigs:
            out["eig"].append(run.all_eigenvalue)
            out["kept"].append(run.kept_counts)
    return out


SWEEP_SEED = 20260512


def sweep_instances(n=512, seed=SWEEP_SEED):
    """The seeded SIAM parameter sweep: U ~ U[0.05, 1.0], eps_d = -U/2 +
    U[-0.1, 0.1], V log-uniform on [0.03, 0.3], Lambda in {2, 2.5, 3}, Nkeep
    in {256, 512, 1024, 2048}, 30-60 Wilson sites (both ends included).  Each
    instance is an rgflowSIAM-form run (examples/rgflowSIAM/main.cpp:27-42):
    the V site, then `nsites` Wilson sites, all eigenvalues per iteration."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        U = float(rng.uniform(0.05, 1.0))
        eps = -0.5 * U + float(rng.uniform(-0.1, 0.1))
        V = float(math.exp(rng.uniform(math.log(0.03), math.log(0.3))))
        lam = float((2.0, 2.5, 3.0)[rng.integers(0, 3)])
        nkeep = int((256, 512, 1024, 2048)[rng.integers(0, 4)])
        nsites = int(rng.integers(30, 61))
        out.append(dict(U=U, eps=eps, V=V, lam=lam, nkeep=nkeep, nsites=nsites))
    return out


def run_flow_batch(engine, instances, keep_eigs=True):
    """RG flows of several SIAM instances (sweep_instances entries: eps, U,
    V, lam, nkeep, nsites) stepped together through the batched API: one
    launch per phase covers the blocks of every run still running, whatever
    its Lambda, Nkeep or length.  Returns per instance the list of
    all_eigenvalue arrays (V site excluded) and kept counts, as run_nrg does."""
    runs = [api.NrgCore(engine, M.spinhalf(p["eps"], p["U"]), M.spinhalf(0.0, 0.0), p["nkeep"])
            for p in instances]
    out = [{"eig": [], "kept": []} for _ in instances]
    try:
        api.batch_add_site(runs, [[p["V"]] * 2 for p in instances], [1.0] * len(runs))
        api.batch_update_state(runs)
        for it in range(max(p["nsites"] for p in instances)):
            act = [k for k, p in enumerate(instances) if it < p["nsites"]]
            rs = [runs[k] for k in act]
            api.batch_add_site(rs, [[M.hopping(it, instances[k]["lam"])] * 2 for k in act],
                               [math.sqrt(instances[k]["lam"]) if it > 0 else 1.0 for k in act])
            api.batch_update_state(rs)
            if keep_eigs:
                for k in act:
                    out[k]["eig"].append(runs[k].all_eigenvalue)
                    out[k]["kept"].append(runs[k].kept_counts)
    finally:
        for r in runs:
            r.close()
    return out


def flow_request(kind, nkeep, nsites, lam, V=None, eps=-0.25, U=0.5, J=0.25):
    """Server.submit keyword arguments of one RG-flow request (all
    eigenvalues per site, no backward pass) for the model families the
    serving mix draws: 'siam' (V site, then Wilson sites; rgflowSIAM form),
    'kondo' (no V site, sqrt(Lambda) rescale from the first site;
    rgflowKondo form, examples/rgflowKondo/main.cpp:20-31) and 'twochannel'
    (four hoppings per site; examples/twoChannelSiam/main.cpp:24-40)."""
    imp, bath = build_models(kind, eps, U, J)
    nops = len(imp.fdag)
    if kind in ("kondo", "zero"):
        t = [[M.hopping(it, lam)] * nops for it in range(nsites)]
        rescale = [math.sqrt(lam)] * nsites
    else:
        t = [[V] * nops] + [[M.hopping(it, lam)] * nops for it in range(nsites)]
        rescale = [1.0] + [math.sqrt(lam) if it > 0 else 1.0 for it in range(nsites)]
    return dict(impurity=imp, bath=bath, nkeep=nkeep, t=np.array(t), rescale=np.array(rescale),
                keep_eigenvalues=True)


SERVING_SEED = 20261204


def serving_mix(n, seed=SERVING_SEED, nkeep_siam=(256, 512, 1024, 2048, 4096),
                nkeep_kondo=(256, 512, 1024, 2048, 4096), nkeep_twochannel=(256, 512, 1024)):
    """The seeded request mix of the serving workload: 60 % SIAM (parameters
    drawn as in the sweep: U ~ U[0.05, 1], eps_d = -U/2 + U[-0.1, 0.1], V
    log-uniform on [0.03, 0.3], Lambda in {2, 2.5, 3}), 25 % Kondo (J
    log-uniform on [0.05, 0.3], Lambda = 2.5), 15 % two-channel SIAM (eps_d =
    -0.3, U = 0.6, Lambda = 4, V ~ U[0.08, 0.15]); 30-50 Wilson sites; Nkeep
    drawn per family from the given sets.  Returns [(family, params)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        u = float(rng.random())
        ns = int(rng.integers(30, 51))
        if u < 0.60:
            U = float(rng.uniform(0.05, 1.0))
            p = dict(kind="siam", U=U, eps=-0.5 * U + float(rng.uniform(-0.1, 0.1)),
                     V=float(math.exp(rng.uniform(math.log(0.03), math.log(0.3)))),
                     lam=float((2.0, 2.5, 3.0)[rng.integers(0, 3)]),
                     nkeep=int(nkeep_siam[rng.integers(0, len(nkeep_siam))]), nsites=ns)
        elif u < 0.85:
            p = dict(kind="kondo", J=float(math.exp(rng.uniform(math.log(0.05), math.log(0.3)))), lam=2.5,
                     nkeep=int(nkeep_kondo[rng.integers(0, len(nkeep_kondo))]), nsites=ns)
        else:
            p = dict(kind="twochannel", eps=-0.3, U=0.6, V=float(rng.uniform(0.08, 0.15)), lam=4.0,
                     nkeep=int(nkeep_twochannel[rng.integers(0, len(nkeep_twochannel))]), nsites=ns)
        out.append(p)
    return out


def mix_request(p):
    """flow_request of one serving_mix entry."""
    return flow_request(p["kind"], p["nkeep"], p["nsites"], p["lam"], V=p.get("V"), eps=p.get("eps", -0.25),
                        U=p.get("U", 0.5), J=p.get("J", 0.25))
