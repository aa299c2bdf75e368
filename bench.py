"""Benchmark: complete SIAM spectral runs per second on one GB300, the mixed-
precision batched engine against the plain FP64 GPU path.

Workload (``--workload``, default ``siam_fdm_nk2048``): the impurity spectral
run eps_d=-0.4, U=0.8, V=0.15, Lambda=2 at Nkeep=2048 over 40 Wilson sites
(``siam_fdm_nk1024``: Nkeep=1024, 50 sites) -- forward NRG with the
d-dagger-chi operators tracked and device-resident snapshots, the T=0 FDM
backward pass (1e5 log bins), log-Gaussian broadening (b=0.6, 100 points per
decade over |w| in [1e-8, 1]) and entropy / specific heat on the 200-point
temperature grid.  One step = ENGINES engines, each driven by its own host
thread, each stepping BATCH runs together (one launch per phase for all
their blocks).  The reference publishes no number for this metric.

  value      : runs/s through the engine, mixed precision, results left on
               the device (every site's eigenvalues still come back to the
               host, as the truncation bookkeeping needs them)
  e2e        : runs/s through the public C-ABI calls a user makes, with the
               per-site all_eigenvalue and the final spectra /
               thermodynamics copied to host buffers inside the timed region
  plain_fp64 : the same steps on the plain FP64 GPU path (warm-up step, then
               timed steps), with its own roofline against a measured FP64
               peak (cuBLAS DGEMM through torch, CUDA events)
  error      : every eigenvalue of every site, the spectral function and
               the thermodynamics of both paths against the reference's own
               outputs for this workload (tests/golden fixtures) and against
               each other
  sweep      : runs/s of a chunk of the seeded 512-instance SIAM sweep
               (mixed Lambda, Nkeep, lengths; RG flows) on both paths
  serving    : the workload's runs as requests to the continuous-batching
               server, seeded Poisson arrivals at 80 % of the batch
               throughput: p50 / p99 latency and served runs/s
  serving_mix: the seeded request mix (60 % SIAM, 25 % Kondo, 15 %
               two-channel RG flows) under a 160 GB admission budget
  roofline   : the dominant kernel, useful work only (an FP64-accurate
               tensor-core product counts 2MNK, not its digit-plane
               products), plus the path-level (F_eig + F_rot) / t
  --impl reference : the reference's CPU algorithm (the numpy port of the
               oracle) on this host's cores, the better of one run on all
               threads and one single-threaded run per core

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload siam_fdm_nk2048|siam_fdm_nk1024]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "siam_fdm_nk2048": dict(kind="siam", nkeep=2048, nsites=40, lam=2.0, eps=-0.4, U=0.8, V=0.15,
                            fixture="ref_siam_fdm_nk2048", thermo_fixture="ref_siam_thermo_nk2048",
                            engines=4, batch=4),
    "siam_fdm_nk1024": dict(kind="siam", nkeep=1024, nsites=50, lam=2.0, eps=-0.4, U=0.8, V=0.15,
                            fixture="ref_c2_siam_fdm_nk1024", thermo_fixture="ref_c2_siam_thermo_nk1024",
                            engines=4, batch=8),
}
WORK = dict(WORKLOADS["siam_fdm_nk2048"])
NAME = "siam_fdm_nk2048"
BATCH = int(os.environ.get("NRG_BENCH_BATCH", "0")) or WORK["batch"]      # runs stepped together per engine
ENGINES = int(os.environ.get("NRG_BENCH_ENGINES", "0")) or WORK["engines"]  # engines (host threads) per step


def log(*a):
    """Progress of the phases on stderr (the result line alone goes to stdout)."""
    print("[bench %.0f s]" % (time.perf_counter() - T0), *a, file=sys.stderr, flush=True)


T0 = time.perf_counter()


def select_workload(name):
    global WORK, NAME, BATCH, ENGINES
    if name not in WORKLOADS:
        raise SystemExit("unknown workload %r (one of %s)" % (name, ", ".join(WORKLOADS)))
    NAME = name
    WORK = dict(WORKLOADS[name])
    BATCH = int(os.environ.get("NRG_BENCH_BATCH", "0")) or WORK["batch"]
    ENGINES = int(os.environ.get("NRG_BENCH_ENGINES", "0")) or WORK["engines"]


def config():
    w = WORK
    return {"workload": NAME, "impurity": "spinhalf(eps_d=%g,U=%g)" % (w["eps"], w["U"]),
            "V": w["V"], "Lambda": w["lam"], "Nkeep": w["nkeep"], "sites": w["nsites"],
            "spectral": "T=0 FDM (the reference's fdmSpectrum is T=0 only), b=0.6, 801 points |w| in [1e-8,1]",
            "thermo": "entropy + C on 200-point T grid",
            "l2": "flushed (256 MiB write) between steps", "runs_per_step": ENGINES * BATCH,
            "engines": ENGINES, "runs_per_engine": BATCH}


def metric():
    return "SIAM runs/s (full FDM spectral run, Nkeep=%d, %d sites), mixed precision" % (
        WORK["nkeep"], WORK["nsites"])


def serving_run(engine, rate, n, seed=2024, max_active=None, workers=None):
    """Seeded Poisson stream of n workload requests at `rate` per second into
    the serving loop (`workers` engines, up to `max_active` runs each);
    latency = submission to completed results."""
    import threading
    import numpy as np
    from nrgplusplus_gb300 import api, workloads
    max_active = BATCH if max_active is None else max_active
    workers = ENGINES if workers is None else workers
    w = WORK
    req = workloads.siam_request(w["nkeep"], w["nsites"], w["lam"], w["V"], eps=w["eps"], U=w["U"],
                                 fdm=True, thermo=True, keep_eigs=False)
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, size=n)
    srv = api.Server(engine, max_active=max_active, workers=workers)
    ids = []

    def arrivals():
        for g in gaps:
            time.sleep(float(g))
            ids.append(srv.submit(**req))

    t0 = time.perf_counter()
    th = threading.Thread(target=arrivals)
    th.start()
    th.join()
    for i in ids:
        srv.wait(i, 3600.0)
        srv.result(i)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"requests": n, "arrival_rate_per_s": rate, "seed": seed, "max_active_per_worker": max_active,
            "workers": workers,
            "runs_per_s": st["completed"] / wall, "p50_latency_s": st["p50_latency_s"],
            "p99_latency_s": st["p99_latency_s"], "mean_latency_s": st["mean_latency_s"],
            "max_active_seen": int(st["max_active_seen"]), "failed": int(st["failed"]),
            "arrivals": "Poisson, seeded; every request the full workload run (FDM + thermodynamics)"}


def serving_mix_run(engine, n, seed=None, max_active=None, workers=None, budget=160 * 10 ** 9, load=0.8):
    """The serving mix: 2 n seeded requests (60 % SIAM, 25 % Kondo, 15 %
    two-channel RG flows; workloads.serving_mix) into a server with an HBM
    admission budget of `budget` bytes, in two phases on fresh servers:
    the first n submitted at once give the mix's capacity (runs/s); the
    next n arrive as a seeded Poisson stream at `load` x that capacity, and
    their latencies are reported (an arrival rate above the capacity would
    measure queueing, not serving)."""
    import threading
    import numpy as np
    from nrgplusplus_gb300 import api, workloads
    seed = workloads.SERVING_SEED if seed is None else seed
    max_active = BATCH if max_active is None else max_active
    workers = ENGINES if workers is None else workers
    mix = workloads.serving_mix(2 * n, seed)
    reqs = [workloads.mix_request(p) for p in mix]

    def phase(rs, gaps):
        srv = api.Server(engine, max_active=max_active, workers=workers, hbm_budget_bytes=budget)
        ids = []

        def arrivals():
            for g, r in zip(gaps, rs):
                if g > 0:
                    time.sleep(float(g))
                ids.append(srv.submit(**r))

        t0 = time.perf_counter()
        th = threading.Thread(target=arrivals)
        th.start()
        th.join()
        for i in ids:
            srv.wait(i, 3600.0)
            srv.result(i)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return st, wall

    st1, w1 = phase(reqs[:n], [0.0] * n)
    capacity = st1["completed"] / w1
    rate = load * capacity
    gaps = np.random.default_rng(seed + 1).exponential(1.0 / rate, size=n)
    st, wall = phase(reqs[n:], gaps)
    fam = {}
    for p in mix:
        fam.setdefault(p["kind"], []).append(p["nkeep"])
    return {"requests": n, "capacity_runs_per_s": capacity, "capacity_requests": n, "arrival_rate_per_s": rate,
            "load": load, "seed": seed, "hbm_budget_bytes": budget,
            "max_active_per_worker": max_active, "workers": workers,
            "families": {k: {"count": len(v), "nkeep": sorted(set(v))} for k, v in fam.items()},
            "runs_per_s": st["completed"] / wall, "p50_latency_s": st["p50_latency_s"],
            "p99_latency_s": st["p99_latency_s"], "mean_latency_s": st["mean_latency_s"],
            "max_active_seen": int(st["max_active_seen"]), "failed": int(st["failed"]) + int(st1["failed"]),
            "what": "RG flows (all eigenvalues per site) of the seeded mix, 30-50 sites each: capacity from "
                    "the first requests submitted at once, latencies of the next ones arriving at `load` "
                    "x capacity"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def max_over_ranks(values):
    """Element-wise maximum of a list of floats over the ranks of the
    initialised process group (the values unchanged without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def _site_bytes(site):
    """Host bytes of one site description as the C ABI receives it."""
    n = 0
    n += 4 * sum(len(q) for q in site.qnums) + 4 * len(site.energies)
    n += 8 * sum(len(e) for e in site.energies) + 8 * len(site.chi)
    for op in site.fdag:
        for m in op.values():
            n += 12 + 8 * m.size
    return n


def _ops_bytes(ops):
    return sum(20 + 8 * m.size for op in ops for m in op.values())


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region (samples in
    a temporary file, summarised into the result line)."""

    def __init__(self):
        self.p = None
        self.path = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        fd, self.path = tempfile.mkstemp(prefix="nrg_bench_clocks_", suffix=".csv")
        self.f = os.fdopen(fd, "w")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.close()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = max(mx, float(f[2]))
                except ValueError:
                    continue
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                    "sw_power_cap"), f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        except OSError:
            pass
        finally:
            try:
                os.remove(self.path)
            except OSError:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def one_run(engine, e2e, batch=None, collect=False):
    """One engine's share of a step: `batch` complete spectral runs stepped
    together (one launch per phase for all their blocks), then their backward
    passes shell by shell (the FDM of every run in one batched call per
    shell).  With e2e the caller-visible results are copied to host buffers as
    a user of the API would read them.  Returns (host-to-device bytes of the
    inputs, device-to-host bytes of the results, outputs of run 0 when
    `collect`: every site's all_eigenvalue, the histograms, the broadened
    spectral functions, entropy and specific heat)."""
    import numpy as np
    from nrgplusplus_gb300 import api, workloads
    from nrgplusplus_gb300 import models as M
    w = WORK
    B = BATCH if batch is None else batch
    lam = w["lam"]
    runs = [api.NrgCore(engine, M.spinhalf(w["eps"], w["U"]), M.spinhalf(0.0, 0.0), w["nkeep"])
            for _ in range(B)]
    datas = [api.NrgData(r) for r in runs]
    api.batch_add_site(runs, [[w["V"]] * 2] * B, [1.0] * B)
    ops = [api.OperatorSet(r, M.d_dag_chi()) for r in runs]
    for r, o in zip(runs, ops):
        api.update_system_operator(r, o)
    api.batch_update_state(runs)
    d2h = 0
    min_it = [0] * B
    got = {"eig": []} if collect else None
    for it in range(w["nsites"]):
        api.batch_add_site(runs, [[M.hopping(it, lam)] * 2] * B, [math.sqrt(lam) if it > 0 else 1.0] * B)
        api.update_system_operator_batch(runs, ops)
        for k in range(B):
            if runs[k].checkHigherEnergyDiscarded():
                datas[k].saveCurrentData(ops[k])
            else:
                min_it[k] += 1
        api.batch_update_state(runs)
        if e2e:
            d2h += sum(r.all_eigenvalue.nbytes for r in runs)
        if collect:
            got["eig"].append(runs[0].all_eigenvalue)
    om = np.logspace(-8, 0, 801)
    fs = [api.FdmSpectrum(r, 2) for r in runs]
    ths = [api.FdmThermodynamics(r, workloads.temperature_grid()) for r in runs]
    cnt = [r.nrg_iterations_cnt for r in runs]
    for it in range(w["nsites"], min(min_it), -1):
        todo = [k for k in range(B) if it > min_it[k]]
        for k in todo:
            cnt[k] -= 1
            datas[k].loadCurrentData(cnt[k])
        sc = lam ** (-(it - 1.0) / 2.0)
        api.fdm_calc_batch([fs[k] for k in todo], [sc] * len(todo))
        for k in todo:
            ths[k].calcThermodynamics(sc)
    for k, run in enumerate(runs):
        spec = fs[k].saveFinalData()
        A = [engine.broaden(spec["GreenFnEnergyPoints"], spec[key][ip], om, 0.6)
             for key in ("GreenFnPositiveWeight", "GreenFnNegativeWeight") for ip in range(2)]
        tdat = ths[k].saveFinalData()
        d2h += spec["GreenFnPositiveWeight"].nbytes * 2 + sum(a.nbytes for a in A)
        d2h += tdat["entropy"].nbytes * 2
        if collect and k == 0:
            got.update(spectra=A, energies=spec["GreenFnEnergyPoints"], entropy=tdat["entropy"],
                       cv=tdat["specificHeat"], omegas=om)
        fs[k].close()
        ths[k].close()
        ops[k].close()
        run.close()
    imp, bath = M.spinhalf(w["eps"], w["U"]), M.spinhalf(0.0, 0.0)
    h2d = B * (_site_bytes(imp) + _site_bytes(bath) + _ops_bytes(M.d_dag_chi())
               + 8 * (w["nsites"] + 1) * 3 + 8 * len(workloads.temperature_grid()))
    return h2d, d2h, got


def step(engines, e2e, batch=None, collect=False):
    """One bench step: every engine runs one_run in its own host thread
    (ctypes releases the GIL inside each C-ABI call).  Returns the summed
    (h2d, d2h) bytes and engine 0's collected outputs; re-raises the first
    error of any thread."""
    import threading
    res, errs = [None] * len(engines), []

    def drive(k):
        try:
            res[k] = one_run(engines[k], e2e, batch, collect and k == 0)
        except BaseException as x:  # noqa: BLE001 - re-raised below
            errs.append(x)

    ths = [threading.Thread(target=drive, args=(k,)) for k in range(len(engines))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    if errs:
        raise errs[0]
    return sum(r[0] for r in res), sum(r[1] for r in res), res[0][2]


# ------------------------------------------------------------ CPU baseline
def _cpu_sample(work, sites):
    """One bounded sample of the workload on the numpy port of the oracle:
    the V site, `sites` Wilson sites with d-dagger-chi tracked, then the FDM
    and thermodynamics backward passes over the shells it produced.
    Returns its wall time in seconds."""
    from oracle.nrg_oracle import siam_run
    from nrgplusplus_gb300 import models as M
    t0 = time.perf_counter()
    siam_run(M.spinhalf(work["eps"], work["U"]), M.spinhalf(0, 0), work["nkeep"], sites, work["lam"],
             V=work["V"], track_ops=M.d_dag_chi(), fdm=True, thermo=True, full_fdag=False)
    return time.perf_counter() - t0


class CpuBaseline:
    """The reference's algorithm on this host's cores, in the two modes of a
    throughput baseline: one run at a time on all BLAS threads ("one"), and
    one single-threaded run per core at once ("per_core", a spawn-started
    process pool, so it may start after the GPU is in use).  A sample runs
    the first `sites` of the workload's Wilson sites and its backward passes;
    runs/s counts it as sites/nsites of a run (per-site cost is flat once the
    truncation starts and lower before, so the extrapolation favours the
    CPU)."""

    def __init__(self, sites):
        self.sites = max(1, min(sites, WORK["nsites"]))
        self.cores = cpu_cores()
        self.pool = None

    def _pool(self):
        if self.pool is None:
            import multiprocessing as mp
            keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
            old = {k: os.environ.get(k) for k in keys}
            for k in keys:
                os.environ[k] = "1"
            try:
                self.pool = mp.get_context("spawn").Pool(self.cores)
                self.pool.starmap(_cpu_sample, [(dict(WORK, nkeep=16), 1)] * self.cores)  # imports done
            finally:
                for k, v in old.items():
                    if v is None:
                        os.environ.pop(k, None)
                    else:
                        os.environ[k] = v
        return self.pool

    def measure(self, mode):
        """(runs/s, wall seconds) of one sample in `mode`."""
        frac = self.sites / WORK["nsites"]
        t0 = time.perf_counter()
        if mode == "one":
            _cpu_sample(WORK, self.sites)
            n = 1
        else:
            self._pool().starmap(_cpu_sample, [(WORK, self.sites)] * self.cores)
            n = self.cores
        wall = time.perf_counter() - t0
        return n * frac / wall, wall

    def best(self):
        """Both modes once; the better one's line."""
        r1, w1 = self.measure("one")
        r2, w2 = self.measure("per_core")
        mode, v, w = ("one", r1, w1) if r1 >= r2 else ("per_core", r2, w2)
        return {"value": v, "unit": "runs/s", "cores": self.cores,
                "kind": "port", "mode": mode,
                "modes": {"one_run_all_threads": r1, "one_run_per_core": r2},
                "sample": "numpy port of the reference (LAPACK syevd + BLAS dgemm), the workload's "
                          "first %d of %d Wilson sites with operator tracking, FDM and thermodynamics "
                          "backward passes, counted as %d/%d of a run; better of one run on all threads "
                          "(%.2f runs/s) and %d single-threaded runs at once (%.2f runs/s); %.1f s"
                          % (self.sites, WORK["nsites"], self.sites, WORK["nsites"], r1, self.cores, r2, w)}

    def close(self):
        if self.pool is not None:
            self.pool.terminate()
            self.pool.join()
            self.pool = None


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def reference_arm(args):
    """--impl reference: the CPU algorithm on this host, steps of one bounded
    sample each, in whichever mode the warm-up found faster."""
    ws, rank = _dist()
    if rank != 0:
        return 0
    cb = CpuBaseline(args.cpu_sites)
    try:
        r = {"one": cb.measure("one")[0], "per_core": cb.measure("per_core")[0]}
        mode = max(r, key=r.get)
        for _ in range(max(0, args.warmup - 2)):
            cb.measure(mode)
        walls, vals = [], []
        for _ in range(args.steps):
            v, w = cb.measure(mode)
            vals.append(v)
            walls.append(w)
    finally:
        cb.close()
    t = sum(walls) / len(walls)
    v = sum(vals) / len(vals)
    sample = ("numpy port of the reference (LAPACK syevd + BLAS dgemm): per step %s, each the first %d of %d "
              "Wilson sites of the workload with operator tracking, FDM and thermodynamics backward passes, "
              "counted as %d/%d of a run; mode chosen by the warm-up (one run on all threads %.3f runs/s, "
              "%d single-threaded runs at once %.3f runs/s)"
              % ("one run on all host threads" if mode == "one" else "%d single-threaded runs at once" % cb.cores,
                 cb.sites, WORK["nsites"], cb.sites, WORK["nsites"], r["one"], cb.cores, r["per_core"]))
    line = {"impl": "reference", "metric": metric(), "value": v, "unit": "runs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (model parameters only)", "config": config(),
            "cpu_baseline": {"value": v, "unit": "runs/s", "cores": cb.cores, "threads_mode": mode,
                             "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- rooflines
FP32_PEAK_TFLOPS = 80.5   # nominal: 152 SMs x 128 FP32 lanes x 2 flops x 2.07 GHz


def _measured(key, fallback):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key]), "of measured (MEASURED_PEAKS.json %s)" % key
    except (OSError, KeyError, ValueError):
        return fallback, "of fallback (%s)" % key


def measure_fp32_peak():
    """FP32 (CUDA-core) peak of this GPU: cuBLAS SGEMM 8192^3 with TF32 off,
    measured like measure_fp64_peak."""
    import torch
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        return measure_fp64_peak(torch.float32)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def measure_fp64_peak(dtype=None):
    """FP64 peak of this GPU: cuBLAS DGEMM 8192^3 through torch.matmul, best
    of 5 after 2 warm-ups, CUDA events on torch's stream (2 N^3 flops)."""
    import torch
    dtype = dtype or torch.float64
    n = 8192
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    c = torch.empty_like(a)
    for _ in range(2):
        torch.matmul(a, b, out=c)
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def kernel_models(fp64_peak, fp32_peak=None):
    """Per kernel: (bound, peak, unit, multiplier from the recorded work to the
    unit's numerator, peak source, per-launch work definition)."""
    fp32, fp32_src = ((fp32_peak, "of measured (cuBLAS SGEMM 8192^3, TF32 off, in this run)") if fp32_peak
                      else (FP32_PEAK_TFLOPS, "of nominal GB300 FP32"))
    bf16, bf16_src = _measured("bf16_tflops_sustained", 1700.0)
    hbm, hbm_src = _measured("hbm_gbs", 6800.0)
    fp64 = ("fp64", fp64_peak, "TFLOP/s", 1e-12, "of measured (cuBLAS DGEMM 8192^3 in this run)",
            "2MNK per GEMM contribution / (10/3) n^3 per eigensolved block")
    return {
        "k_gemm_f64": fp64,
        "k_eig_f64": fp64,
        "k_eig_bi_f32": ("fp32", fp32, "TFLOP/s", 1e-12, fp32_src,
                         "(4/3) n^3 per block (Householder reduction)"),
        "k_reflect": ("fp32", fp32, "TFLOP/s", 1e-12, fp32_src,
                      "2 n^3 per block (Householder reflectors applied to the tridiagonal eigenvectors)"),
        "k_gemm_oz": ("tensor", bf16, "TFLOP/s", 1e-12, bf16_src,
                      "useful work: 2MNK per FP64-accurate product; the bf16 digit-plane products it "
                      "takes are reported apart (tensor_pipe)"),
        "k_split": ("hbm", hbm, "GB/s", 1e-9, hbm_src,
                    "bytes: 8 (max pass) + 8 (digit pass) read + 16 written per element"),
        "k_oa_update": ("hbm", hbm, "GB/s", 1e-9, hbm_src, "bytes: S, G read + E written, 24 per element"),
    }


# DRAM bytes (read + write) per launch measured with ncu on one engine's
# 4-run batch of the Nkeep = 2048 workload, cold cache (mean over the
# batch's launches; profiles/launches_siam_fdm_nk2048_engine.md)
MEASURED_TRAFFIC = {"k_gemm_oz": 435.5e6, "k_eig_bi_f32": 177.1e6, "k_oa_update": 156.3e6,
                    "k_reflect": 101.0e6, "k_split": 300.8e6}


def kernel_profile(engine, batch=None):
    """One extra engine batch with per-kernel CUDA events on the engine
    stream; returns ({kernel: (ms, work, launches)}, work counters)."""
    engine.set_profiling(True)
    engine.kernel_times()
    engine.work_counters(reset=True)
    one_run(engine, e2e=False, batch=batch)
    kt = engine.kernel_times()
    wc = engine.work_counters(reset=True)
    engine.set_profiling(False)
    return kt, wc


def _roofline(name, ms, work, n, models):
    bound, peak, unit, mult, src, per = models[name]
    achieved = work * mult / (ms * 1e-3) if ms > 0 else 0.0
    return {"bound": bound, "kernel": name, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak if peak else None, "traffic": MEASURED_TRAFFIC.get(name),
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
            "peak_source": src, "launches": n, "ms_total": ms, "per_launch": per}


def roofline_from(kt, wc, fp64_peak, fp32_peak=None):
    """Roofline of the kernel with the largest share of the batch, every
    modelled kernel's own line, and the tensor-pipe view of k_gemm_oz."""
    models = kernel_models(fp64_peak, fp32_peak)
    known = {k: v for k, v in kt.items() if k in models}
    top = max(known.items(), key=lambda kv: kv[1][0])
    rf = _roofline(top[0], *top[1], models)
    rf["all"] = {k: {"achieved": round(r["achieved"], 3), "unit": r["unit"], "frac": round(r["frac"], 5),
                     "bound": r["bound"], "ms": round(v[0], 3), "traffic": r["traffic"]}
                 for k, v in known.items() for r in [_roofline(k, *v, models)]}
    if "k_gemm_oz" in kt and kt["k_gemm_oz"][0] > 0 and wc.get("tc_useful"):
        ms = kt["k_gemm_oz"][0]
        bf16 = models["k_gemm_oz"][1]
        pipe = wc["tc_bf16"] / (ms * 1e-3) / 1e12
        rf["tensor_pipe"] = {"kernel": "k_gemm_oz", "bf16_tflops": pipe, "frac_of_bf16_peak": pipe / bf16,
                             "digit_plane_products_per_useful": wc["tc_bf16"] / wc["tc_useful"],
                             "note": "bf16 tensor-pipe work the FP64-accurate products took; not useful work"}
    return rf


# ------------------------------------------------------------------ errors
def _eig_tol(N, lam):
    """Eigenvalue tolerance of the parity tests (tests/parity.py eig_tol):
    1e-10 absolute in iteration units until the reference's own FP64 noise,
    which grows like Lambda^(N/2) along the flow, exceeds it."""
    return max(1e-10, 1e-14 * lam ** (N / 2.0))


def _compare(got, ref_eigs, ref_spectra, ref_entropy, ref_cv, T):
    import numpy as np
    lam = WORK["lam"]
    eabs, eover, emax_site = 0.0, 0.0, 0
    for i, (a, b) in enumerate(zip(got["eig"], ref_eigs)):
        if a.size != b.size:
            return {"eig_count_mismatch_at_site": i}
        d = float(np.abs(a - b).max()) if a.size else 0.0
        if d > eabs:
            eabs, emax_site = d, i
        eover = max(eover, d / _eig_tol(i, lam))
    spec = 0.0
    for a, b in zip(got["spectra"], ref_spectra):
        spec = max(spec, float(np.abs(a - b).max() / np.abs(b).max()))
    m = T >= 2.6e-7
    return {"eig_max_abs": eabs, "eig_max_abs_site": emax_site, "eig_max_over_tol": eover,
            "eig_values_compared": int(sum(a.size for a in got["eig"])),
            "spectral_max_rel": spec,
            "entropy_max_abs": float(np.abs(got["entropy"] - ref_entropy).max()),
            "cv_max_rel_T_ge_2.6e-7": float(np.max(np.abs(got["cv"][m] - ref_cv[m]) / np.abs(ref_cv[m])))}


def output_errors(engine, got_mixed, got_fp64):
    """Both paths' outputs of one run against the reference's outputs for the
    same workload (tests/golden fixtures, generated from the reference
    compiled from its own sources) and against each other."""
    import numpy as np
    from nrgplusplus_gb300 import workloads
    gold = os.path.join(ROOT, "tests", "golden")
    fx = np.load(os.path.join(gold, WORK["fixture"] + ".npz"))
    th = np.load(os.path.join(gold, WORK["thermo_fixture"] + ".npz"))
    T = workloads.temperature_grid()
    eigs = [fx["eig%d" % i] for i in range(WORK["nsites"])]
    e = got_mixed["energies"]
    om = got_mixed["omegas"]
    spectra = []
    for key in ("Positive", "Negative"):
        for ip in range(2):
            h = np.zeros(100000)
            h[fx["GreenFn%sWeight%d_idx" % (key, ip)]] = fx["GreenFn%sWeight%d_val" % (key, ip)]
            spectra.append(engine.broaden(e, h, om, 0.6))
    out = {"vs_reference": {}, "tolerances": {
        "eig": "|dE| <= max(1e-10, 1e-14 Lambda^(N/2)) per site N (the reference's own FP64 noise); "
               "the headline target is 1e-9", "spectral": "1e-6 of the maximum", "entropy": "1e-8"}}
    for name, got in (("mixed", got_mixed), ("fp64", got_fp64)):
        if got:
            out["vs_reference"][name] = _compare(got, eigs, spectra, th["entropy"], th["specificHeat"], T)
    if got_mixed and got_fp64:
        out["mixed_vs_fp64"] = _compare(got_mixed, got_fp64["eig"], got_fp64["spectra"], got_fp64["entropy"],
                                        got_fp64["cv"], T)
    return out


# ------------------------------------------------------------------- sweep
def sweep_pass(engines, count):
    """The first `count` instances of the seeded 512-instance sweep, spread
    over the engines (greedy by Nkeep^2 x sites), each engine stepping its
    share as one heterogeneous batch in its own host thread.  Two passes:
    the first warms the engines on the sweep's block-size histograms (the
    autotuner times its candidates on the first launch of each); the second
    is timed.  Returns its wall time in seconds."""
    _sweep_once(engines, count)
    return _sweep_once(engines, count)


def _sweep_once(engines, count):
    import threading
    from nrgplusplus_gb300 import workloads
    inst = workloads.sweep_instances()[:count]
    order = sorted(range(len(inst)), key=lambda k: -inst[k]["nkeep"] ** 2 * inst[k]["nsites"])
    load, share = [0.0] * len(engines), [[] for _ in engines]
    for k in order:
        j = min(range(len(engines)), key=lambda x: load[x])
        share[j].append(inst[k])
        load[j] += inst[k]["nkeep"] ** 2 * inst[k]["nsites"]
    errs = []

    def drive(j):
        try:
            if share[j]:
                workloads.run_flow_batch(engines[j], share[j], keep_eigs=True)
        except BaseException as x:  # noqa: BLE001 - re-raised below
            errs.append(x)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=drive, args=(j,)) for j in range(len(engines))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for e in engines:
        e.sync()
    wall = time.perf_counter() - t0
    if errs:
        raise errs[0]
    return wall


# -------------------------------------------------------------------- main
def timed_steps(engines, k, e2e, barrier, flush, batch=None):
    """k timed steps (L2 flushed before each, barrier + sync on both sides);
    returns (seconds per step list, h2d, d2h, algorithmic work of the steps)."""
    times, h2d, d2h = [], 0, 0
    for e in engines:
        e.work_counters(reset=True)
    for _ in range(k):
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        h2d, d2h, _ = step(engines, e2e=e2e, batch=batch)
        for e in engines:
            e.sync()
        barrier()
        times.append(time.perf_counter() - t0)
    work = {"F_eig": 0.0, "F_rot": 0.0}
    for e in engines:
        wc = e.work_counters(reset=True)
        work["F_eig"] += wc["F_eig"]
        work["F_rot"] += wc["F_rot"]
    return times, h2d, d2h, work


def path_roofline(work, seconds, peak, peak_src, pipe):
    """Path level: (F_eig + F_rot) / t over the timed steps."""
    a = (work["F_eig"] + work["F_rot"]) / seconds / 1e12
    return {"achieved": a, "unit": "TFLOP/s", "peak": peak, "frac": a / peak, "peak_source": peak_src,
            "pipe": pipe, "F_eig_per_run": None, "F_rot_per_run": None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--workload", default="siam_fdm_nk2048", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-sites", type=int, default=0,
                    help="Wilson sites of one bounded CPU-baseline sample (default: per workload)")
    ap.add_argument("--e2e-steps", type=int, default=3, help="timed steps of the e2e measurement")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the plain FP64 comparator")
    ap.add_argument("--fp64-batch", type=int, default=0,
                    help="runs per engine of the FP64 comparator (default: as the mixed path)")
    ap.add_argument("--sweep-runs", type=int, default=32,
                    help="instances of the seeded sweep timed on both paths (0: skip)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparator")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--serving-requests", type=int, default=24)
    ap.add_argument("--mix-requests", type=int, default=16,
                    help="requests of the serving mix, half for its capacity, half timed (0: skip)")
    ap.add_argument("--sites", type=int, default=0,
                    help="Wilson sites per run (default: the workload's; fewer only for profiling captures)")
    args = ap.parse_args()
    select_workload(args.workload)
    if not args.cpu_sites:
        args.cpu_sites = 14 if WORK["nkeep"] >= 2048 else 20
    reduced = bool(args.sites) and args.sites != WORK["nsites"]
    if reduced:
        WORK["nsites"] = args.sites
    if args.impl == "reference":
        return reference_arm(args)
    import torch
    from nrgplusplus_gb300 import api
    from nrgplusplus_gb300.build import build
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    build(verbose=False)
    fp64_peak = measure_fp64_peak()
    fp32_peak = measure_fp32_peak()
    engines = [api.Engine(api.PREC_MIXED, device=local) for _ in range(ENGINES)]
    engine = engines[0]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    log("workload", NAME, "engines", ENGINES, "runs per engine", BATCH,
        "FP64 peak %.3f TFLOP/s, FP32 peak %.1f TFLOP/s" % (fp64_peak, fp32_peak))
    got_mixed = None
    for w in range(max(1, args.warmup)):
        _, _, got = step(engines, e2e=False, collect=(w == 0 and not reduced))
        got_mixed = got_mixed or got
    launch_total = lambda: sum(e.launch_count() for e in engines)  # noqa: E731
    l0 = launch_total()
    with ClockSampler() as clk:
        times, _, _, work = timed_steps(engines, args.steps, False, barrier, flush)
        launches = (launch_total() - l0) // args.steps
        e2e_times, h2d, d2h, _ = timed_steps(engines, max(1, args.e2e_steps), True, barrier, flush)
    clocks = clk.summary()
    runs = ENGINES * BATCH
    log("mixed: %d steps, %.3f s/step; e2e %.3f s/step" % (len(times), sum(times) / len(times),
                                                          sum(e2e_times) / len(e2e_times)))
    tsum, esum = max_over_ranks([sum(times), sum(e2e_times)])
    per = tsum / args.steps
    value = ws * runs / per
    e2e_v = ws * runs / (esum / len(e2e_times))
    bf16, bf16_src = _measured("bf16_tflops_sustained", 1700.0)
    path = path_roofline(work, tsum, bf16, bf16_src + "; the pipe that carries the bulk of the mixed path",
                         "bf16 tensor")
    path["F_eig_per_run"] = work["F_eig"] / (runs * args.steps)
    path["F_rot_per_run"] = work["F_rot"] / (runs * args.steps)
    path["frac_of_fp64_peak"] = path["achieved"] / fp64_peak
    kt, wc = kernel_profile(engine)
    rf = roofline_from(kt, wc, fp64_peak, fp32_peak)
    log("kernels (ms per engine batch):", {k: round(v[0], 1) for k, v in kt.items()})
    rf["path"] = path
    fallbacks = sum(e.fallback_count() for e in engines)
    hbm_peak = sum(e.memory()[1] for e in engines)
    sweep = None
    if args.sweep_runs > 0 and not reduced:
        sweep = {"instances": args.sweep_runs, "of": 512, "seed": "workloads.SWEEP_SEED",
                 "what": "RG flows (all eigenvalues per site) of the first instances of the seeded sweep, "
                         "one heterogeneous batch per engine; the second of two passes is timed"}
        t = sweep_pass(engines, args.sweep_runs)
        sweep["mixed_runs_per_s"] = args.sweep_runs / t
        log("sweep mixed: %.3f runs/s" % sweep["mixed_runs_per_s"])
    for e in engines[1:]:
        e.close()
    serving = mix = None
    if not args.no_serving and not reduced:
        serving = serving_run(engine, 0.8 * runs / per, args.serving_requests)
        log("serving:", serving)
        if args.mix_requests > 0:
            mix = serving_mix_run(engine, max(2, args.mix_requests // 2))
            log("serving mix:", mix)
    engine.close()
    plain, got_fp64 = None, None
    if not args.no_fp64:
        e64s = [api.Engine(api.PREC_FP64, device=local) for _ in range(ENGINES)]
        b64 = args.fp64_batch or BATCH
        _, _, got_fp64 = step(e64s, e2e=False, batch=b64, collect=not reduced)  # warm-up
        t64s, _, _, work64 = timed_steps(e64s, max(1, args.fp64_steps), False, barrier, flush, batch=b64)
        t64 = max_over_ranks([sum(t64s)])[0] / len(t64s)
        log("fp64: %.3f s/step" % t64)
        kt64, wc64 = kernel_profile(e64s[0], b64)
        rf64 = roofline_from(kt64, wc64, fp64_peak, fp32_peak)
        p64 = path_roofline(work64, sum(t64s), fp64_peak, "of measured (cuBLAS DGEMM 8192^3 in this run)",
                            "fp64")
        p64["F_eig_per_run"] = work64["F_eig"] / (ENGINES * b64 * len(t64s))
        p64["F_rot_per_run"] = work64["F_rot"] / (ENGINES * b64 * len(t64s))
        rf64["path"] = p64
        if sweep is not None:
            sweep["fp64_runs_per_s"] = args.sweep_runs / sweep_pass(e64s, args.sweep_runs)
            sweep["speedup_mixed_over_fp64"] = sweep["mixed_runs_per_s"] / sweep["fp64_runs_per_s"]
            log("sweep fp64: %.3f runs/s" % sweep["fp64_runs_per_s"])
        for e in e64s:
            e.close()
        runs64 = ENGINES * b64
        plain = {"value": ws * runs64 / t64, "unit": "runs/s", "ms_per_step": t64 * 1e3, "runs_per_step": runs64,
                 "steps": len(t64s), "warmup": 1, "speedup_mixed_over_fp64": value / (ws * runs64 / t64),
                 "fp64_peak_tflops": fp64_peak, "fp64_peak_source": "cuBLAS DGEMM 8192^3 via torch.matmul, "
                 "best of 5, CUDA events (this run)", "roofline": rf64,
                 "kernels_ms_per_engine_batch": {k: round(v[0], 3) for k, v in kt64.items()}}
    errors = None
    if got_mixed is not None:
        e0 = api.Engine(api.PREC_FP64, device=local)
        errors = output_errors(e0, got_mixed, got_fp64)
        e0.close()
        log("errors:", errors)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cb = CpuBaseline(args.cpu_sites)
        try:
            cpu = cb.best()
        finally:
            cb.close()
        log("cpu:", cpu)
    if rank == 0:
        cfg = dict(config(), precision_path="mixed: FP32 block solve + FP64-accurate refinement on "
                                            "tensor cores; FP64 for refinement, rescale and Boltzmann sums")
        if reduced:
            cfg["workload"] += "_reduced_for_profiling"
            cfg["sites"] = WORK["nsites"]
        line = {"metric": metric(), "value": value, "unit": "runs/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
                "data": "synthetic (model parameters of the workload; no dataset)",
                "config": cfg, "gpu_launches": launches, "fp64_fallback_blocks": fallbacks,
                "hbm_peak_bytes": hbm_peak,
                "e2e": {"value": e2e_v, "unit": "runs/s", "steps": len(e2e_times), "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "plain_fp64": plain, "error": errors, "sweep": sweep, "serving": serving, "serving_mix": mix,
                "roofline": rf,
                "kernels_ms_per_engine_batch": {k: round(v[0], 3) for k, v in kt.items()},
                "kernels_profiled": "one engine's %d-run batch alone, per-kernel CUDA events on its stream"
                                    % BATCH,
                "cpu_baseline": cpu, "clocks": clocks}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def _close_engines():
    """Close every engine still open (after a failure, before the CUDA
    context goes away at exit)."""
    import gc
    try:
        from nrgplusplus_gb300 import api
    except Exception:
        return
    for obj in gc.get_objects():
        if isinstance(obj, api.Engine):
            try:
                obj.close()
            except Exception:
                pass


if __name__ == "__main__":
    try:
        rc = main()
    except BaseException:
        _close_engines()
        raise
    sys.exit(rc)
