"""Benchmark: complete SIAM FDM runs per second on one GB300.

One run = the spectral workload (eps_d=-0.4, U=0.8, V=0.15, Lambda=2,
Nkeep=1024, 50 Wilson sites): forward NRG with the d-dagger-chi operators
tracked and device-resident snapshots, the T=0 FDM backward pass (binning
into 1e5 log bins), log-Gaussian broadening (b=0.6, 100 points per decade
over |w| in [1e-8, 1]) and entropy / specific heat on the 200-point
temperature grid.  One step = ENGINES engines, each driven by its own host
thread, each stepping RUNS_PER_ENGINE runs together (batched launches); the
engines' streams overlap one engine's host work with another's kernels.
The reference publishes no number for this metric.

  value : runs/s through the engine, results left on the device
  e2e   : runs/s through the public C-ABI calls a user makes, with the
          per-site all_eigenvalue and the final spectra / thermodynamics
          copied to host buffers inside the timed region
  --impl reference : the reference's CPU algorithm (the numpy port of the
          oracle) timed on this host's cores on the same workload
  serving : the same runs as requests to the continuous-batching server
          (nrg_server_*), seeded Poisson arrivals at 80 % of the measured
          batch throughput: p50 / p99 request latency and served runs/s

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORK = dict(kind="siam", nkeep=1024, nsites=50, lam=2.0, eps=-0.4, U=0.8, V=0.15)
BATCH = int(os.environ.get("NRG_BENCH_BATCH", "8"))  # runs stepped together per engine
ENGINES = int(os.environ.get("NRG_BENCH_ENGINES", "4"))  # engines (host threads) per step
CONFIG = {"workload": "siam_fdm_spectral_c2", "impurity": "spinhalf(eps_d=-0.4,U=0.8)",
          "V": 0.15, "Lambda": 2.0, "Nkeep": 1024, "sites": 50, "T": 1e-6,
          "spectral": "T=0 FDM, b=0.6, 801 points |w| in [1e-8,1]",
          "thermo": "entropy + C on 200-point T grid",
          "l2": "flushed (256 MiB write) between steps", "runs_per_step": ENGINES * BATCH,
          "engines": ENGINES, "runs_per_engine": BATCH}
METRIC = "SIAM runs/s (full FDM spectral run, Nkeep=1024, 50 sites)"


def serving_run(engine, rate, n, seed=2024, max_active=BATCH, workers=ENGINES):
    """Seeded Poisson stream of n workload requests at `rate` per second into
    the serving loop (`workers` engines, up to `max_active` runs each);
    latency = submission to completed results."""
    import threading
    import numpy as np
    from nrgplusplus_gb300 import api, workloads
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
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def one_run(engine, e2e, batch=None):
    """One step: `batch` complete spectral runs stepped together (one launch
    per phase for all their blocks), then each run's backward passes.  With
    e2e the caller-visible results are copied to host buffers as a user of
    the API would read them.  Returns the host-to-device bytes of the inputs
    (models, tracked operators, hoppings, temperatures) and the device-to-host
    bytes of the results of the step."""
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
    om = np.logspace(-8, 0, 801)
    # backward passes of all runs shell by shell, the FDM of every run in one
    # batched call per shell (the thermodynamics are host sums)
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
        fs[k].close()
        ths[k].close()
        ops[k].close()
        run.close()
    imp, bath = M.spinhalf(w["eps"], w["U"]), M.spinhalf(0.0, 0.0)
    h2d = B * (_site_bytes(imp) + _site_bytes(bath) + _ops_bytes(M.d_dag_chi())
               + 8 * (w["nsites"] + 1) * 3 + 8 * len(workloads.temperature_grid()))
    return h2d, d2h


def step(engines, e2e, batch=None):
    """One bench step: every engine runs one_run in its own host thread
    (ctypes releases the GIL inside each C-ABI call).  Returns the summed
    (h2d, d2h) bytes; re-raises the first error of any thread."""
    import threading
    res, errs = [None] * len(engines), []

    def drive(k):
        try:
            res[k] = one_run(engines[k], e2e, batch)
        except BaseException as x:  # noqa: BLE001 - re-raised below
            errs.append(x)

    ths = [threading.Thread(target=drive, args=(k,)) for k in range(len(engines))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    if errs:
        raise errs[0]
    return sum(r[0] for r in res), sum(r[1] for r in res)


def time_oracle_run(max_sites):
    """The oracle port on this host's cores: the same workload, forward sites
    capped at max_sites (bounded sample)."""
    from oracle.nrg_oracle import siam_run
    from nrgplusplus_gb300 import models as M
    w = WORK
    t0 = time.perf_counter()
    siam_run(M.spinhalf(w["eps"], w["U"]), M.spinhalf(0, 0), w["nkeep"], max_sites, w["lam"],
             V=w["V"], track_ops=M.d_dag_chi(), fdm=True, thermo=False, full_fdag=True)
    return time.perf_counter() - t0


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def reference_arm(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    times = []
    sites = WORK["nsites"]
    for _ in range(args.warmup if args.warmup < 1 else 1):
        time_oracle_run(4)
    for _ in range(args.steps):
        times.append(time_oracle_run(sites))
    t = sum(times) / len(times)
    v = 1.0 / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "runs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (model parameters only)", "config": CONFIG,
            "cpu_baseline": {"value": v, "unit": "runs/s", "cores": cpu_cores(), "kind": "port",
                             "sample": "full workload per step (numpy restatement of the reference, "
                                       "LAPACK syevd + BLAS dgemm, all host threads)"},
            "e2e": {"value": v, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# nominal per-GPU peaks for the pipes MEASURED_PEAKS.json does not cover
FP64_PEAK_TFLOPS = 1.25   # GB300 FP64 (vector and tensor) dense
FP32_PEAK_TFLOPS = 80.5   # 152 SMs x 128 FP32 lanes x 2 flops x 2.07 GHz


def _measured(key, fallback):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key]), "of measured (MEASURED_PEAKS.json %s)" % key
    except (OSError, KeyError, ValueError):
        return fallback, "of fallback (%s)" % key


def kernel_models():
    """Per kernel: (bound, peak, unit, multiplier from the recorded work to the
    unit's numerator, peak source, per-launch work definition)."""
    bf16, bf16_src = _measured("bf16_tflops_sustained", 1700.0)
    hbm, hbm_src = _measured("hbm_gbs", 6800.0)
    fp64 = ("fp64", FP64_PEAK_TFLOPS, "TFLOP/s", 1e-12, "nominal GB300 FP64",
            "2MNK per GEMM contribution / (10/3) n^3 per eigensolved block")
    return {
        "k_gemm_f64": fp64,
        "k_eig_f64": fp64,
        "k_eig_bi_f32": ("fp32", FP32_PEAK_TFLOPS, "TFLOP/s", 1e-12, "nominal GB300 FP32",
                         "(4/3) n^3 per block (Householder reduction)"),
        "k_reflect": ("fp32", FP32_PEAK_TFLOPS, "TFLOP/s", 1e-12, "nominal GB300 FP32",
                      "2 n^3 per block (Householder reflectors applied to the tridiagonal eigenvectors)"),
        "k_gemm_oz": ("tensor", bf16, "TFLOP/s", 1e-12, bf16_src,
                      "bf16 tensor flops: 2MNK per digit-plane product (36 products per FP64-accurate "
                      "product with 8 planes, 15 with the 5 planes of the first refinement step)"),
        "k_split": ("hbm", hbm, "GB/s", 1e-9, hbm_src,
                    "bytes: 8 (max pass) + 8 (digit pass) read + 16 written per element"),
        "k_oa_update": ("hbm", hbm, "GB/s", 1e-9, hbm_src, "bytes: S, G read + E written, 24 per element"),
    }


# DRAM bytes (read + write) per launch measured with ncu on one engine's full
# 8-run step (mean over its 869 launches; summary and command under profiles/)
MEASURED_TRAFFIC = {"k_gemm_oz": 221.0e6}


def kernel_profile(engine):
    """One extra run with per-kernel CUDA events on the engine stream."""
    engine.set_profiling(True)
    engine.kernel_times()
    one_run(engine, e2e=False)
    kt = engine.kernel_times()
    engine.set_profiling(False)
    return kt


def _roofline(name, ms, work, n, models):
    bound, peak, unit, mult, src, per = models[name]
    achieved = work * mult / (ms * 1e-3) if ms > 0 else 0.0
    return {"bound": bound, "kernel": name, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak if peak else None, "traffic": MEASURED_TRAFFIC.get(name),
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
            "peak_source": src,
            "launches": n, "ms_total": ms, "per_launch": per}


def roofline_from(kt):
    """Roofline of the kernel with the largest share of the step, plus every
    modelled kernel's own line."""
    models = kernel_models()
    known = {k: v for k, v in kt.items() if k in models}
    top = max(known.items(), key=lambda kv: kv[1][0])
    rf = _roofline(top[0], *top[1], models)
    rf["all"] = {k: {"achieved": round(r["achieved"], 2), "unit": r["unit"], "frac": round(r["frac"], 4),
                     "bound": r["bound"], "ms": round(v[0], 3)}
                 for k, v in known.items() for r in [_roofline(k, *v, models)]}
    return rf


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--cpu-sites", type=int, default=50,
                    help="forward sites of the bounded CPU-baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparator")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serving-requests", type=int, default=64)
    ap.add_argument("--sites", type=int, default=50,
                    help="Wilson sites per run (50 = the workload; fewer only for profiling captures)")
    args = ap.parse_args()
    if args.sites != WORK["nsites"]:
        WORK["nsites"] = args.sites
        CONFIG["sites"] = args.sites
        CONFIG["workload"] += "_reduced_for_profiling"
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
    engines = [api.Engine(api.PREC_MIXED, device=local) for _ in range(ENGINES)]
    engine = engines[0]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step(engines, e2e=False)
    times, d2h = [], 0
    launch_total = lambda: sum(e.launch_count() for e in engines)  # noqa: E731
    l0 = launch_total()
    os.makedirs(os.path.join(ROOT, "gpurun_out"), exist_ok=True)
    with ClockSampler(os.path.join(ROOT, "gpurun_out", "bench_clocks.csv")) as clk:
        for _ in range(args.steps):
            flush.zero_()
            barrier()
            t0 = time.perf_counter()
            step(engines, e2e=False)
            for e in engines:
                e.sync()
            barrier()
            times.append(time.perf_counter() - t0)
        launches = (launch_total() - l0) // args.steps
        e2e_times = []
        for _ in range(args.steps):
            flush.zero_()
            barrier()
            t0 = time.perf_counter()
            h2d, d2h = step(engines, e2e=True)
            for e in engines:
                e.sync()
            barrier()
            e2e_times.append(time.perf_counter() - t0)
    runs = ENGINES * BATCH
    tsum, esum = max_over_ranks([sum(times), sum(e2e_times)])
    per = tsum / args.steps
    value = ws * runs / per
    e2e_v = ws * runs / (esum / args.steps)
    kt = kernel_profile(engine)
    rf = roofline_from(kt)
    fallbacks = sum(e.fallback_count() for e in engines)
    hbm_peak = sum(e.memory()[1] for e in engines)
    for e in engines[1:]:
        e.close()
    serving = None
    if not args.no_serving:
        serving = serving_run(engine, 0.8 * runs / per, args.serving_requests)
    engine.close()
    plain = None
    if not args.no_fp64:
        e64s = [api.Engine(api.PREC_FP64, device=local) for _ in range(ENGINES)]
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        step(e64s, e2e=False)
        for e in e64s:
            e.sync()
        barrier()
        t64 = time.perf_counter() - t0
        for e in e64s:
            e.close()
        plain = {"value": ws * runs / t64, "unit": "runs/s", "ms_per_step": t64 * 1e3,
                 "speedup_mixed_over_fp64": value / (ws * runs / t64)}
    cpu = None
    if rank == 0 and ws == 1:
        sites = max(1, min(args.cpu_sites, WORK["nsites"]))
        tc = time_oracle_run(sites)
        cpu = {"value": 1.0 / tc, "unit": "runs/s (of the sample)", "cores": cpu_cores(), "kind": "port",
               "sample": "numpy oracle, same model, forward %d of 50 sites + FDM backward "
                         "(%.1f s); runs/s of that truncated run" % (sites, tc)}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "runs/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
                "data": "synthetic (model parameters of the workload; no dataset)",
                "config": dict(CONFIG, precision_path="mixed: FP32 block solve + FP64-accurate refinement"),
                "gpu_launches": launches,
                "fp64_fallback_blocks": fallbacks,
                "hbm_peak_bytes": hbm_peak,
                "e2e": {"value": e2e_v, "unit": "runs/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "serving": serving, "plain_fp64": plain, "roofline": rf,
                "kernels_ms_per_engine_batch": {k: round(v[0], 3) for k, v in kt.items()},
                "kernels_profiled": "one engine's %d-run batch alone, per-kernel CUDA events on its stream"
                                    % BATCH,
                "cpu_baseline": cpu, "clocks": clk.summary()}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
