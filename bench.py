"""Benchmark: CLV pattern-node updates/s of the pruning likelihood on GB300.

Workload: full post-order lnL evaluations of a 128-taxon Yule tree (branch
lengths Exp(mean 0.05)) over 100,000 sites simulated under GTR+Gamma4
(alpha 0.5, Dirichlet-drawn parameters), compressed to unique patterns;
every evaluation recomputes every internal CL (127 node updates x P
patterns).  One "step" is a batch of --batch such evaluations (default 256,
the work of 256 model proposals), so that the timed region lasts seconds and
the clock sampler sees it.  The headline form is the FP32-scaled plan
walker; the plain FP64 path is measured beside it on the same plan.

  value      updates/s of the FP32 form, device-timed with CUDA events over
             K steps of back-to-back runs (inputs resident in HBM; each run
             writes ~0.6 GB of CLs, more than L2, so no extra flush is needed)
  e2e        the same metric through the public API (Lik.lnL with a full
             re-plan each step: host planning, program upload from pinned
             memory, kernels, result read-back)
  roofline   plan-walker kernel: algorithmic bytes per launch / event time,
             against MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the FP64 oracle CxLikExecute on the host cores (reference
             build when present, else this repository's port)
  batched    the same tree under 32 sets of exchangeabilities in one
             persistent batched launch (the work of 32 chains' proposals)

``--impl reference`` times the reference's CPU implementation on the same
workload instead and prints its own line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "gtr_gamma4_128taxa_100ksites_full_lnL",
            "ntaxa": 128, "nsites": 100000, "mean_brlen": 0.05,
            "alpha": 0.5, "ncat": 4, "seed": 20261203}
METRIC = "CLV pattern-node updates/s (FP32-scaled form, full post-order lnL)"
UNIT = "updates/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Dist:
    """Barrier and max-reduce across replica ranks (gloo; one GPU each)."""

    def __init__(self):
        self.ws, self.rank = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.out = None
        self.path = None

    def start(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(prefix="crux_gb300_clocks_", suffix=".csv")
        self.out = os.fdopen(fd, "w")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader",
                 "-lms", "100"], stdout=self.out, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
            self.out.close()
            os.unlink(self.path)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = [r.split(",") for r in open(self.path).read().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1].split()[0]))
                smax.append(float(r[2].split()[0]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if "Active" in v and "Not" not in v:
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def make_case():
    from crux_gb300 import synth
    w = WORKLOAD
    return synth.Case(w["ntaxa"], w["nsites"], w["mean_brlen"], w["seed"],
                      alpha=w["alpha"], ncat=w["ncat"])


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def profile_traffic(name):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def autotune(lib, prec, args, lik=None, liks=None, lanes=True):
    """Pick the walker's launch shape (tile, threads per pattern, patterns
    per thread, stack budget, op lanes) by timing the candidates on this
    workload; ``--shape`` fixes it instead.  `lanes` False keeps one op lane
    (MC3 and the server run the batched walker, which has one).  Returns
    the shape with how it was chosen."""
    from crux_gb300 import tune
    if args.shape:
        tune.set_shape(lib, *args.shape)
        t, g, p, b = args.shape[:4]
        n = args.shape[4] if len(args.shape) > 4 else 1
        return {"tile": t, "tpp": g, "ppt": p, "budget": b, "lanes": n,
                "source": "--shape"}
    if liks is not None:
        r = tune.tune_batch(liks, prec, iters=3,
                            shapes=tune.candidates(
                                prec, tune.active_components(liks[0]),
                                budgets=(12 << 10, 24 << 10, 48 << 10),
                                lanes=(1,)))
    else:
        r = tune.tune_plan(lik, prec, iters=10,
                           shapes=None if lanes else tune.candidates(
                               prec, tune.active_components(lik), lanes=(1,)))
    best = dict(r["best"])
    top = sorted(r["table"], key=lambda x: x["ms"])
    per_tpp = {}
    for x in top:
        key = str(x["tpp"])
        if x["ppt"] != 1:
            key += "/ppt%d" % x["ppt"]
        if x["lanes"] != 1:
            key += "/lanes%d" % x["lanes"]
        per_tpp.setdefault(key, [x["tile"], x["budget"], x["ms"]])
    best.update(source="autotuned", candidates=len(r["table"]),
                worst_ms=top[-1]["ms"], best_per_tpp=per_tpp)
    return best


def batched_measure(gpu, case, nevals, oracle=None):
    """The bench tree under `nevals` different GTR exchangeabilities (the
    work of as many chains' proposals) in one persistent batched launch
    (crux_gb300.batch.Batch): pattern-node updates/s of the walk, its
    roofline by algorithmic bytes, and two of the lnLs against the FP64
    oracle.  The shape is tuned on this batch."""
    import numpy as np
    from crux_gb300 import tune
    from crux_gb300.batch import Batch
    aln = case.alignment()
    rng = np.random.default_rng(WORKLOAD["seed"] + 1)
    rates = [[float(x) for x in rng.dirichlet(np.ones(6)) * 6] for _ in range(nevals)]
    liks = []
    for r in rates:
        lk = case.lik(lib=gpu, precision="fp32", alignment=aln)
        lk.setRclass(0, [0, 1, 2, 3, 4, 5], r)
        lk.prepare_plan()
        liks.append(lk)
    tr = tune.tune_batch(liks, "fp32", iters=3,
                         shapes=tune.candidates("fp32", 4,
                                                budgets=(0, 12 << 10, 24 << 10),
                                                lanes=(1,)))
    b = Batch(liks, "fp32")
    got = b.run()
    b.time(3)
    t = b.time(20)
    info = b.info()
    b.close()
    peaks = measured_peaks()
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = info["alg_bytes"] / (t["walk_ms"] / 1e3) / 1e9
    out = {"evals_per_launch": nevals,
           "value": info["updates"] / (t["walk_ms"] / 1e3), "unit": UNIT,
           "walk_ms": t["walk_ms"], "ms_per_run": t["ms_per_run"],
           "ms_per_eval": t["walk_ms"] / nevals,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                        "unit": "GB/s", "frac": achieved / hbm},
           "shape": dict(tr["best"])}
    if oracle is not None:
        err = 0.0
        for i in (0, nevals - 1):
            lo = case.lik(lib=oracle, alignment=case.alignment())
            lo.setRclass(0, [0, 1, 2, 3, 4, 5], rates[i])
            want = lo.lnL()
            err = max(err, abs(got[i] - want) / abs(want))
        out["rel_err_vs_fp64_oracle"] = err
    del liks
    return out


def cpu_run(lib, case, aln, steps, threads, min_s=0.0):
    """Time full-plan FP64 evaluations of the oracle: at least `steps`, and
    more until `min_s` seconds of CxLikExecute have run.  Returns
    (updates/s, seconds, updates, evaluations)."""
    from crux_gb300 import synth
    lik = case.lik(lib=lib, alignment=aln)
    lik.lnL()
    t = 0.0
    ups = 0
    n = 0
    while n < steps or t < min_s:
        n += 1
        lik.lik.invalidate = True
        lik._prep(None)
        t0 = time.perf_counter()
        lib.CxLikExecute(ctypes.byref(lik.lik))
        t += time.perf_counter() - t0
        ups += synth.nnodes_updates(lik)
    return ups / t, t, ups, n


def load_cpu_oracle():
    from oracle import oracle
    lib = oracle.load_ref()
    threads = os.cpu_count() or 1
    if lib is not None:
        oracle.ref_threaded(lib)
        threads = oracle.ref_ncpus(lib)
        return lib, "reference", threads
    lib = oracle.load_port()
    lib.port_set_threads(threads)
    return lib, "port", threads


def tree128_config(npat, nops, ws):
    """The tree128 workload's config; both arms print exactly this."""
    return dict(WORKLOAD, patterns=npat, node_updates_per_eval=nops,
                parallelism="replicas" if ws > 1 else "single",
                l2_flush="inputs>L2 (each evaluation writes all %d internal "
                         "CLs of %d patterns)" % (nops, npat))


REF_EVALS_PER_STEP = 8


def run_reference(args, dist):
    """--impl reference: the reference's CPU path on the host cores.  Each
    step is a bounded sample of REF_EVALS_PER_STEP full-tree evaluations of
    CxLikExecute; planning (the Python restatement of Lik._plan, outside
    the timed calls) never maps this package's GPU library."""
    if dist.rank != 0:
        dist.close()
        return
    from crux_gb300 import synth
    lib, kind, threads = load_cpu_oracle()
    case = make_case()
    aln = case.alignment()
    cpu_run(lib, case, aln, max(args.warmup, 1) * REF_EVALS_PER_STEP, threads)
    rate, secs, ups, nev = cpu_run(lib, case, aln,
                                   args.steps * REF_EVALS_PER_STEP, threads)
    probe = case.lik(lib=lib, alignment=aln)
    probe.prepare_plan()
    nops = synth.nnodes_updates(probe) // int(probe.lik.mschars)
    line = {"metric": METRIC, "impl": "reference", "value": rate, "unit": UNIT,
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Yule tree, GTR+G4 simulation)",
            "config": tree128_config(aln.nchars, nops, dist.ws),
            "evals_per_step": REF_EVALS_PER_STEP,
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads,
                             "kind": kind,
                             "sample": "%d steps x %d full-tree FP64 lnL "
                                       "evaluations (%.1f s)" %
                                       (args.steps, REF_EVALS_PER_STEP, secs)},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    dist.close()


def run_ours(args, dist):
    from crux_gb300 import _native, synth
    from crux_gb300.plan import Plan
    gpu = _native.load()
    case = make_case()

    from crux_gb300 import tune
    res = {}
    for prec in ((args.precision,) if args.profile else ("fp32", "fp64")):
        lik = case.lik(lib=gpu, precision=prec)
        lnl_first = lik.lnL()
        lik.lik.invalidate = True
        lik._prep(None)
        shape = autotune(gpu, prec, args, lik=lik)
        plan = Plan(lik, prec)
        info = plan.info()
        plan.time(max(args.warmup, 3))
        dist.barrier()
        clocks = Clocks()
        if prec == "fp32":
            clocks.start()
        t = plan.time(args.steps * args.batch)
        ck = clocks.stop() if prec == "fp32" else None
        ms = dist.max(t["ms_per_run"])
        res[prec] = {"lik": lik, "plan": plan, "info": info, "t": t,
                     "ms": ms, "clocks": ck, "lnL": t["lnL"],
                     "lnL_first": lnl_first, "shape": shape,
                     "plan_shape": plan.shape()}

    if args.profile:
        for p in res.values():
            p["plan"].close()
        print(json.dumps({"profile_run": True, "precision": args.precision,
                          "ms_per_run": res[args.precision]["ms"]}))
        return

    # End to end through the public API: full re-plan + lnL each run, with
    # the FP32 form's tuned shape.  One step is --batch evaluations, as in
    # the device-timed leg.
    sh = res["fp32"]["shape"]
    tune.set_shape(gpu, sh["tile"], sh["tpp"], sh["ppt"], sh["budget"],
                   sh["lanes"])
    lik = res["fp32"]["lik"]
    for _ in range(max(args.warmup, 3)):
        lik.lik.invalidate = True
        lik.lnL()
    dist.barrier()
    e2e_runs = args.steps * args.batch
    t0 = time.perf_counter()
    for _ in range(e2e_runs):
        lik.lik.invalidate = True
        lik.lnL()
    e2e_s = dist.max((time.perf_counter() - t0) / e2e_runs)
    # The host planner alone (Lik._plan of a full re-plan), reported apart
    # from the device work as the reference's planner is.
    t0 = time.perf_counter()
    for _ in range(50):
        lik.lik.invalidate = True
        lik._prep(None)
    planner_ms = (time.perf_counter() - t0) / 50 * 1e3
    lik.lik.invalidate = True
    lik.lnL()
    h2d, d2h = ctypes.c_size_t(), ctypes.c_size_t()
    gpu.cxgLikLastIo(ctypes.byref(h2d), ctypes.byref(d2h))
    # The drop-in call Crux itself makes (Lik.pyx:1699-1712): CxLikExecute
    # on host CL structs, every site lnL and stripe sum written back to host
    # memory, then summed on the host.  It computes in the reference's
    # precision (the plain FP64 form).
    ld = case.lik(lib=gpu, alignment=case.alignment(), dropin=True)
    for _ in range(max(args.warmup, 3)):
        ld.lik.invalidate = True
        ld.lnL()
    dropin_runs = args.steps * 8
    t0 = time.perf_counter()
    for _ in range(dropin_runs):
        ld.lik.invalidate = True
        dropin_lnl = ld.lnL()
    dropin_s = dist.max((time.perf_counter() - t0) / dropin_runs)
    dh2d, dd2h = ctypes.c_size_t(), ctypes.c_size_t()
    gpu.cxgLikLastIo(ctypes.byref(dh2d), ctypes.byref(dd2h))
    nops = res["fp32"]["info"]["nops"]
    npat = int(res["fp32"]["lik"].lik.mschars)

    info = res["fp32"]["info"]
    ws = dist.ws
    value = info["updates"] * ws / (res["fp32"]["ms"] / 1e3)
    e2e = info["updates"] * ws / e2e_s
    kern_ms = res["fp32"]["t"]["kernel_ms"]
    peaks = measured_peaks()
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = info["alg_bytes"] / (kern_ms / 1e3) / 1e9
    traffic = profile_traffic("walk_kernel_fp32_128taxa_100ksites.md")

    # Oracle check of both forms (FP64 oracle on the same plan).
    cpu = None
    check = {}
    if dist.rank == 0 and not args.no_cpu:
        lib, kind, threads = load_cpu_oracle()
        aln = case.alignment()
        rate, secs, ups, nev = cpu_run(lib, case, aln, args.cpu_steps,
                                       threads, min_s=args.cpu_seconds)
        want = case.lik(lib=lib, alignment=case.alignment()).lnL()
        check = {p: abs(res[p]["lnL"] - want) / abs(want) for p in res}
        check["dropin_fp64"] = abs(dropin_lnl - want) / abs(want)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": "%d full-tree FP64 lnL evaluations (%.1f s)" %
                         (nev, secs)}
        if kind == "port" and threads > 1:
            # The same on one core, over a shorter bounded sample.
            lib.port_set_threads(1)
            r1, s1, _, n1 = cpu_run(lib, case, aln, 1, 1,
                                    min_s=args.cpu_seconds / 3)
            lib.port_set_threads(threads)
            cpu["single_core"] = {
                "value": r1, "sample": "%d evaluations (%.1f s)" % (n1, s1)}

    if dist.rank == 0:
        fp64 = res["fp64"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["fp32"]["ms"] * args.batch,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Yule tree, GTR+G4 simulation)",
            "config": tree128_config(npat, nops, ws),
            "evals_per_step": args.batch,
            "walker_shape": res["fp32"]["shape"],
            "walker_shape_fp64": fp64["shape"],
            "e2e": {"value": e2e, "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d.value) * args.batch,
                    "d2h_bytes_per_step": int(d2h.value) * args.batch,
                    "evals_per_step": args.batch,
                    "ms_per_eval": e2e_s * 1e3,
                    "planner_ms_per_eval": planner_ms,
                    "api": "Lik.lnL (cxgLikExecuteLnL), FP32-scaled form"},
            "e2e_dropin": {"value": info["updates"] * ws / dropin_s,
                           "unit": UNIT,
                           "h2d_bytes_per_eval": int(dh2d.value),
                           "d2h_bytes_per_eval": int(dd2h.value),
                           "ms_per_eval": dropin_s * 1e3,
                           "api": "CxLikExecute with host siteLnL/stripeLnL "
                                  "(plain FP64 form)"},
            "gpu_launches": args.steps * args.batch * info["kernels_per_run"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic,
                         "traffic_source": "committed ncu summary "
                                           "profiles/walk_kernel_fp32_128taxa_"
                                           "100ksites.md (not measured in "
                                           "this run)",
                         "peak_source": "measured" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "clocks": res["fp32"]["clocks"],
            "fp64_plain": {
                "value": info["updates"] * ws / (fp64["ms"] / 1e3),
                "ms_per_step": fp64["ms"] * args.batch,
                "kernel_ms": fp64["t"]["kernel_ms"],
                "alg_bytes": fp64["info"]["alg_bytes"]},
            "fp32_over_fp64": fp64["ms"] / res["fp32"]["ms"],
            "kernel_ms": kern_ms,
            "rel_err_vs_fp64_oracle": check,
        }
        for p in res.values():
            p["plan"].close()
        if args.batched_evals > 0:
            line["batched"] = batched_measure(
                gpu, case, args.batched_evals, None if args.no_cpu else lib)
        if not args.no_sub:
            # Bounded MC3 and serving records on the same run (each under
            # its own clock sampler).  MC3 tunes its walker shape on its own
            # generations; the server takes the tree's tuned shapes.
            shapes = {"fp32": res["fp32"]["shape"], "fp64": res["fp64"]["shape"]}
            line["mc3"] = mc3_measure(
                MC3["mc3"], args.sub_mc3_gens, args.sub_mc3_gens64,
                args=args, oracle=None if args.no_cpu else lib,
                check_every=1000, seq_gens=args.sub_mc3_gens64)
            line["serve"] = serve_measure(args.sub_serve_datasets,
                                          args.sub_serve_rates, 2.0,
                                          shapes=shapes)
        print(json.dumps(line), flush=True)
    else:
        for p in res.values():
            p["plan"].close()
    dist.close()


BATCH = {"workload": "batch256_logu_taxa16-512_sites500-50000_gtr_gamma4",
         "jobs": 256, "taxa": [16, 512], "sites": [500, 50000],
         "mean_brlen": 0.1, "alpha": 0.5, "seed": 20261204}


def make_batch_cases(n=None):
    """The batched workload: jobs with log-uniform taxon and site counts,
    each simulated under GTR+G4 with its own Dirichlet draws."""
    import numpy as np
    from crux_gb300 import synth
    rng = np.random.default_rng(BATCH["seed"])
    out = []
    for j in range(n or BATCH["jobs"]):
        nt = synth.log_uniform_int(rng, *BATCH["taxa"])
        ns = synth.log_uniform_int(rng, *BATCH["sites"])
        out.append(synth.Case(nt, ns, BATCH["mean_brlen"],
                              int(rng.integers(1 << 30)), alpha=BATCH["alpha"]))
    return out


def run_batch(args, dist):
    """Batched persistent kernel (FP32 form, one graph launch for all jobs)
    against the same jobs issued one launch per node update in the plain
    FP64 form."""
    from crux_gb300 import _native
    from crux_gb300.batch import Batch
    gpu = _native.load()
    t0 = time.perf_counter()
    cases = make_batch_cases(args.jobs)
    setup_s = time.perf_counter() - t0
    res = {}
    liks = {}
    runs = (("fp32", False),) if args.profile else \
        (("fp32", False), ("fp64", True), ("fp64", False))
    for prec, per_node in runs:
        key = prec + ("_per_node" if per_node else "_batched")
        if prec not in liks:
            liks[prec] = [c.lik(lib=gpu, precision=prec) for c in cases]
            for lk in liks[prec]:
                lk.prepare_plan()
        shape = autotune(gpu, prec, args, liks=liks[prec]) if not per_node \
            else None
        b = Batch(liks[prec], prec, per_node=per_node)
        info = b.info()
        lnls = b.run()
        b.time(max(args.warmup, 3) if not per_node else 1)
        clocks = Clocks()
        if key == "fp32_batched":
            clocks.start()
        t = b.time(args.steps if not per_node else max(1, args.steps // 10))
        ck = clocks.stop() if key == "fp32_batched" else None
        b.close()
        res[key] = {"info": info, "t": t, "lnL": lnls, "clocks": ck,
                    "shape": shape}
    if args.profile:
        print(json.dumps({"profile_run": True, "workload": BATCH["workload"],
                          "jobs": len(cases),
                          "ms_per_run": res["fp32_batched"]["t"]["ms_per_run"]}))
        dist.close()
        return
    check = {}
    if not args.no_cpu:
        from oracle import oracle
        port = oracle.load_port()
        port.port_set_threads(os.cpu_count() or 1)
        for j in range(0, len(cases), max(1, len(cases) // 8)):
            want = cases[j].lik(lib=port).lnL()
            for k, r in res.items():
                e = abs(r["lnL"][j] - want) / abs(want)
                check[k] = max(check.get(k, 0.0), e)
    fb = res["fp32_batched"]
    upd = fb["info"]["updates"]
    peaks = measured_peaks()
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = fb["info"]["alg_bytes"] / (fb["t"]["walk_ms"] / 1e3) / 1e9
    line = {
        "metric": "CLV pattern-node updates/s (batched FP32-scaled form)",
        "value": upd / (fb["t"]["ms_per_run"] / 1e3), "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": fb["t"]["ms_per_run"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": dict(BATCH, jobs=len(cases), updates_per_run=upd,
                       items=fb["info"]["items"], grid=fb["info"]["grid"],
                       setup_s=round(setup_s, 1), walker_shape=fb["shape"],
                       walker_shape_fp64=res["fp64_batched"]["shape"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": None},
        "gpu_launches": args.steps * fb["info"]["launches_per_run"],
        "clocks": fb["clocks"],
        "fp64_per_node": {
            "value": upd / (res["fp64_per_node"]["t"]["ms_per_run"] / 1e3),
            "ms_per_run": res["fp64_per_node"]["t"]["ms_per_run"],
            "launches_per_run": res["fp64_per_node"]["info"]["launches_per_run"]},
        "fp64_batched": {
            "value": upd / (res["fp64_batched"]["t"]["ms_per_run"] / 1e3),
            "ms_per_run": res["fp64_batched"]["t"]["ms_per_run"]},
        "speedup_vs_fp64_per_node":
            res["fp64_per_node"]["t"]["ms_per_run"] / fb["t"]["ms_per_run"],
        "rel_err_vs_fp64_oracle_max": check,
    }
    print(json.dumps(line), flush=True)
    dist.close()


MC3 = {"mc3": {"workload": "mc3_128taxa_100ksites_gtr_gamma4_8chains",
               "ntaxa": 128, "nsites": 100000, "mean_brlen": 0.05,
               "nchains": 8, "heat_delta": 0.1, "seed": 20261205,
               "moves": {"brlen": 2.0, "nni": 1.0, "spr": 1.0, "rates": 1.0,
                         "alpha": 1.0}, "gens": 2000, "check_every": 1000},
       # The reference sampler's default proposal mix (Mc3/__init__.pyx:
       # 255-289): one rate category, no +I, mixtures (here of at most four
       # members), eTBR and polytomy jumps as the topology moves.
       "mc3ref": {"workload": "mc3_128taxa_100ksites_reference_default_moves_8chains",
                  "ntaxa": 128, "nsites": 100000, "mean_brlen": 0.05,
                  "nchains": 8, "heat_delta": 0.1, "seed": 20261208,
                  "ncat": 1, "max_models": 4,
                  "moves": {"weight": 30.0, "freqs": 10.0, "rmult": 10.0,
                            "rate": 30.0, "brlen": 20.0, "etbr": 80.0,
                            "ratejump": 10.0, "polytomyjump": 40.0,
                            "freqjump": 10.0, "mixturejump": 5.0},
                  "gens": 2000, "check_every": 1000},
       "mc3small": {"workload": "mc3_16taxa_1000sites_gtr_gamma4_4chains",
                    "ntaxa": 16, "nsites": 1000, "mean_brlen": 0.1,
                    "nchains": 4, "heat_delta": 0.2, "seed": 20261206,
                    "moves": {"brlen": 1.0, "nni": 1.0}, "gens": 1000,
                    "check_every": 250}}


MC3_WARM = 48


def mc3_measure(w, gens, gens64, shapes=None, args=None, oracle=None,
                check_every=None, seq_gens=None):
    """On-device MC3 on workload `w`: `gens` generations of the FP32 chains
    and `gens64` of the plain FP64 chains from the same seed, each under its
    own clock sampler.  Every `check_every` FP32 generations each chain's
    lnL is checked against the FP64 oracle (`oracle`, a CPU library; None:
    no check).  Over the first `seq_gens` generations both runs must take
    the same accept/reject sequence: their per-chain, per-move accept and
    reject counts are equal and their cold-chain traces agree to 1e-6.
    `shapes`: walker shape per precision (else ``args.shape``, else tuned
    on a few generations of each candidate)."""
    import numpy as np
    from crux_gb300 import _native, synth, tune
    from crux_gb300.mc3 import Mc3
    gpu = _native.load()
    case = synth.Case(w["ntaxa"], w["nsites"], w["mean_brlen"], w["seed"])
    aln = case.alignment()
    check_every = check_every or w["check_every"]
    seq_gens = min(seq_gens or gens64, gens, gens64)
    out = {}
    for prec, ngen in (("fp32", gens), ("fp64", gens64)):
        if ngen <= 0:
            continue
        ncat = w.get("ncat", 4)

        def make():
            return Mc3(case.tree(aln.taxaMap), aln, case.params["rates"],
                       case.params["freqs"], alpha=0.5 if ncat > 1 else None,
                       ncat=ncat, nchains=w["nchains"],
                       heat_delta=w["heat_delta"], seed=w["seed"],
                       moves=w["moves"], precision=prec, graph_gens=16,
                       max_models=w.get("max_models", 1))

        if shapes and prec in shapes:
            sh = shapes[prec]
            tune.set_shape(gpu, sh["tile"], sh["tpp"], sh["ppt"], sh["budget"])
            shape = dict(sh, lanes=1, source=sh.get("source", "given"))
        elif args is not None and args.shape:
            shape = autotune(gpu, prec, args)
        else:
            # Tuned on the MC3 run itself (dirty-path walks, not a full
            # plan): a few generations per candidate.
            r = tune.tune_mc3(gpu, make, prec, gens=32 if prec == "fp32" else 8,
                              warm=8 if prec == "fp32" else 2)
            top = sorted(r["table"], key=lambda x: x["ms"])
            shape = dict(r["best"], source="autotuned on MC3 generations",
                         candidates=len(r["table"]), worst_ms=top[-1]["ms"])
        m = make()
        # The same untimed warm-up in both precisions, so that their
        # generations stay aligned for the accept/reject comparison.
        m.run(MC3_WARM)
        secs, drift, done = 0.0, [], 0
        seq = None
        clocks = Clocks()
        clocks.start()
        while done < ngen:
            step = min(check_every - done % check_every, ngen - done)
            if done < seq_gens < done + step:
                step = seq_gens - done
            secs += m.run(step)
            done += step
            if done == seq_gens:
                st = m.stats()
                seq = {"accepts": st["accepts"], "rejects": st["rejects"],
                       "trace": m.trace(MC3_WARM + seq_gens)[MC3_WARM:]}
            if oracle is not None and prec == "fp32" and \
                    (done % check_every == 0 or done == ngen):
                worst = 0.0
                for i in range(m.nchains):
                    lik, st = m.chain_lik(i, oracle)
                    want = lik.lnL()
                    worst = max(worst, abs(st["lnL"] - want) / abs(want))
                drift.append({"generation": done, "max_rel_err": worst})
        ck = clocks.stop()
        st = m.stats()
        acc, rej = int(st["accepts"].sum()), int(st["rejects"].sum())
        from crux_gb300.mc3 import MOVES
        a_m, r_m = st["accepts"].sum(axis=0), st["rejects"].sum(axis=0)
        by_move = {MOVES[j]: {"accepts": int(a_m[j]), "rejects": int(r_m[j])}
                   for j in range(len(MOVES)) if a_m[j] + r_m[j] > 0}
        out[prec] = {"gens_per_s": ngen / secs, "gens": ngen, "secs": secs,
                     "accept_rate": acc / max(1, acc + rej), "by_move": by_move,
                     "swaps": int(st["swaps"].sum()) // 2,
                     "drift_vs_fp64_oracle": drift, "clocks": ck,
                     "walker_shape": shape, "seq": seq}
        m.close()
    res = {"workload": w["workload"], "config": dict(w, gens=gens,
                                                     patterns=aln.nchars)}
    for prec in out:
        r = dict(out[prec])
        r.pop("seq")
        res[prec] = r
    if "fp32" in out and "fp64" in out and out["fp32"]["seq"] is not None \
            and out["fp64"]["seq"] is not None:
        a, b = out["fp32"]["seq"], out["fp64"]["seq"]
        rel = np.abs(a["trace"] - b["trace"]) / np.abs(b["trace"])
        same = bool(np.array_equal(a["accepts"], b["accepts"]) and
                    np.array_equal(a["rejects"], b["rejects"]) and
                    (rel <= 1e-6).all())
        res["accept_sequence"] = {
            "generations": seq_gens, "same_fp32_fp64": same,
            "max_trace_rel_diff": float(rel.max()),
            "first_trace_divergence": (int(np.argmax(rel > 1e-6))
                                       if (rel > 1e-6).any() else None)}
        res["fp32_over_fp64"] = (out["fp32"]["gens_per_s"] /
                                 out["fp64"]["gens_per_s"])
    return res


def run_mc3(args, dist):
    """On-device MC3: generations/s of the FP32-scaled chains and of the
    plain FP64 chains from the same seed, with every chain's lnL checked
    against the FP64 oracle every `check_every` generations."""
    w = dict(MC3[args.workload])
    if args.chains:
        w["nchains"] = args.chains
    gens = args.gens or w["gens"]
    oracle = None
    if not args.no_cpu:
        oracle, _, _ = load_cpu_oracle()
    if args.profile:
        r = mc3_measure(w, gens, 0, args=args)
        print(json.dumps({"profile_run": True, "workload": w["workload"],
                          "nchains": w["nchains"],
                          "gens_per_s": r["fp32"]["gens_per_s"]}))
        dist.close()
        return
    r = mc3_measure(w, gens, gens, args=args, oracle=oracle)
    f32, f64 = r["fp32"], r["fp64"]
    line = {
        "metric": "MC3 generations/s (FP32-scaled chains, on device)",
        "value": f32["gens_per_s"], "unit": "generations/s", "n_gpus": 1,
        "steps": gens, "warmup": MC3_WARM,
        "ms_per_step": 1e3 * f32["secs"] / gens, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": r["config"],
        "fp64_plain_gens_per_s": f64["gens_per_s"],
        "fp32_over_fp64": r["fp32_over_fp64"],
        "accept_rate": f32["accept_rate"], "swaps": f32["swaps"],
        "moves": f32["by_move"],
        "drift_vs_fp64_oracle": f32["drift_vs_fp64_oracle"],
        "accept_sequence": r["accept_sequence"],
        "walker_shape": f32["walker_shape"],
        "walker_shape_fp64": f64["walker_shape"],
        "clocks": f32["clocks"], "clocks_fp64": f64["clocks"],
    }
    print(json.dumps(line), flush=True)
    dist.close()


DIRTY = {"workload": "dirty64_gtr_gamma4_inv_64taxa_10ksites",
         "ntaxa": 64, "nsites": 10000, "mean_brlen": 0.05, "alpha": 0.5,
         "ncat": 4, "pinv": 0.2, "gap_frac": 0.005, "recomputes": 10000,
         "rescale": [0.5, 2.0], "rescale_of": "generated length",
         "seed": 20261208}


def run_dirty(args, dist):
    """A full lnL, then dirty-path lnLs after random single-branch rescales,
    each through the public Lik.lnL call (planning included).  A rescale
    sets one branch to its generated length x U(0.5, 2): compounding the
    factors instead is a random walk with positive drift in log length that
    saturates the tree within a few thousand steps, where the +I
    component's P(0) = V V^-1 (exact only to rounding) dominates sites of
    likelihood below ~1e-16 and no two FP64 eigensolvers agree.  The FP32
    form and the plain FP64 form replay the same rescales; so does the FP64
    oracle on the host cores, which checks every lnL and is timed as the
    CPU baseline."""
    import numpy as np
    from crux_gb300 import _native, synth
    from crux_gb300._abi import STEP_DTYPE, ComputeI, ComputeL
    from crux_gb300.plan import Plan
    w = DIRTY
    n = args.gens or w["recomputes"]
    warm = max(args.warmup, 3)
    gpu = _native.load()
    case = synth.Case(w["ntaxa"], w["nsites"], w["mean_brlen"], w["seed"],
                      alpha=w["alpha"], ncat=w["ncat"], pinv=w["pinv"],
                      gap_frac=w["gap_frac"])
    aln = case.alignment()
    rng = np.random.default_rng(w["seed"])
    nedge = 2 * w["ntaxa"] - 3
    moves = [(int(rng.integers(nedge)), float(rng.uniform(*w["rescale"])))
             for _ in range(warm + n)]

    def replay(lik, count_updates=False):
        edges = lik.tree.edges
        base = [x.length for x in edges]
        vals, ups = [lik.lnL()], 0
        t0 = None
        for i, (e, f) in enumerate(moves):
            if i == warm:
                t0 = time.perf_counter()
            edges[e].length = base[e] * f
            vals.append(lik.lnL())
            if count_updates and i >= warm:
                st = np.frombuffer(lik._steps, dtype=STEP_DTYPE)[:lik.nsteps]
                ups += int(np.isin(st["variant"], (ComputeL, ComputeI)).sum())
        return vals, time.perf_counter() - t0, ups

    out = {}
    for prec in ("fp32", "fp64"):
        lik = case.lik(lib=gpu, precision=prec, alignment=aln)
        lik.prepare_plan()
        shape = autotune(gpu, prec, args, lik=lik)
        lik = case.lik(lib=gpu, precision=prec, alignment=aln)
        clocks = Clocks()
        if prec == "fp32":
            clocks.start()
        vals, secs, _ = replay(lik)
        ck = clocks.stop() if prec == "fp32" else None
        # Node updates per recompute, counted on an untimed replay of the
        # same rescales (the same dirty paths).
        _, _, nodes = replay(case.lik(lib=gpu, precision=prec, alignment=aln),
                             count_updates=True)
        # Device time of one dirty path: the next rescale's plan, rerun.
        lik.tree.edges[0].length *= 1.25
        lik.prepare_plan(full=False)
        plan = Plan(lik, prec)
        plan.time(5)
        dev = plan.time(50)
        plan.close()
        out[prec] = {"vals": vals, "secs": secs, "nodes": nodes,
                     "shape": shape, "clocks": ck, "device": dev}
    cpu, err = None, {}
    if not args.no_cpu:
        lib, kind, threads = load_cpu_oracle()
        lo = case.lik(lib=lib, alignment=case.alignment())
        want, secs, _ = replay(lo)
        want = np.array(want)
        for prec in ("fp32", "fp64"):
            got = np.array(out[prec]["vals"])
            err[prec] = float(np.max(np.abs(got - want) / np.abs(want)))
        cpu = {"value": n / secs, "unit": "recomputes/s", "cores": threads,
               "kind": kind,
               "sample": "the same %d rescales and dirty-path lnLs, "
                         "planning included (%.1f s)" % (n, secs)}
    f32, f64 = out["fp32"], out["fp64"]
    npat = aln.nchars
    line = {
        "metric": "dirty-path lnL recomputes/s through Lik.lnL "
                  "(FP32-scaled form)",
        "value": n / f32["secs"], "unit": "recomputes/s", "n_gpus": 1,
        "steps": n, "warmup": warm, "ms_per_step": 1e3 * f32["secs"] / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": dict(w, recomputes=n, patterns=npat,
                       walker_shape=f32["shape"],
                       walker_shape_fp64=f64["shape"]),
        "updates_per_s": f32["nodes"] * npat / f32["secs"],
        "mean_nodes_per_recompute": f32["nodes"] / n,
        "device_ms_per_dirty_path": f32["device"]["ms_per_run"],
        "fp64_plain": {"value": n / f64["secs"],
                       "updates_per_s": f64["nodes"] * npat / f64["secs"],
                       "device_ms_per_dirty_path": f64["device"]["ms_per_run"]},
        "fp32_over_fp64": f64["secs"] / f32["secs"],
        "cpu_baseline": cpu,
        "max_rel_err_vs_fp64_oracle": err,
        "lnL_checked": len(f32["vals"]) if err else 0,
        "clocks": f32["clocks"],
    }
    print(json.dumps(line), flush=True)
    dist.close()


COMPACT = {"workload": "compact_simulated_gtr_gamma4",
           "shapes": [[128, 100000], [1024, 200000]], "mean_brlen": 0.05,
           "gap_frac": 0.005, "seed": 20261209}


def run_compact(args, dist):
    """Pattern compression (Alignment.compact) of simulated alignments:
    sites/s of the GPU path (cxgCompact, host arrays in and out) against
    the host restatement, with the outputs compared bit for bit."""
    import numpy as np
    from crux_gb300 import _native, synth
    from crux_gb300 import compact as gc
    from crux_gb300.alignment import Alignment, CTMatrix
    gpu = _native.load()
    out = []
    shapes = [args.compact_shape] if args.compact_shape else COMPACT["shapes"]
    for ntaxa, nsites in shapes:
        case = synth.Case(ntaxa, nsites, COMPACT["mean_brlen"], COMPACT["seed"],
                          gap_frac=COMPACT["gap_frac"])
        raw = Alignment(CTMatrix(case.fasta))
        for _ in range(max(args.warmup, 1)):
            gc.compact(raw, gpu)
        reps = max(1, args.steps // 4)
        t0 = time.perf_counter()
        for _ in range(reps):
            rows, freqs, masks = gc.compact(raw, gpu)
        g_s = (time.perf_counter() - t0) / reps
        h = Alignment(CTMatrix(case.fasta))
        t0 = time.perf_counter()
        h.compact()
        h_s = time.perf_counter() - t0
        out.append({"ntaxa": ntaxa, "nsites": nsites, "patterns": int(len(freqs)),
                    "gpu_s": g_s, "host_s": h_s,
                    "gpu_sites_per_s": nsites / g_s, "host_sites_per_s": nsites / h_s,
                    "bit_exact": bool(np.array_equal(rows, h.rows) and
                                      np.array_equal(freqs, h.freqs))})
    line = {
        "metric": "pattern compression sites/s (GPU, host arrays in and out)",
        "value": out[-1]["gpu_sites_per_s"], "unit": "sites/s", "n_gpus": 1,
        "steps": max(1, args.steps // 4), "warmup": max(args.warmup, 1),
        "ms_per_step": 1e3 * out[-1]["gpu_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded)", "config": dict(COMPACT, shapes=shapes), "shapes": out,
    }
    print(json.dumps(line), flush=True)
    dist.close()


SERVE = {"workload": "serve_poisson_logu_taxa8-1024_sites200-200000",
         "datasets": 40, "taxa": [8, 1024], "sites": [200, 200000],
         "pinv_prob": 0.3, "mc3_prob": 0.2, "mc3_gens": 10,
         "rates": [100, 500, 1000, 2000, 5000], "seconds_per_rate": 2.0,
         "resident_datasets": True, "seed": 20261207}


def make_serve_pool(n):
    import numpy as np
    from crux_gb300 import synth
    from crux_gb300.serve import LNL, PreparedRequest
    rng = np.random.default_rng(SERVE["seed"])
    pool = []
    for j in range(n):
        nt = synth.log_uniform_int(rng, *SERVE["taxa"])
        ns = synth.log_uniform_int(rng, *SERVE["sites"])
        pinv = 0.2 if rng.random() < SERVE["pinv_prob"] else 0.0
        case = synth.Case(nt, ns, 0.1, int(rng.integers(1 << 30)), pinv=pinv)
        pool.append(PreparedRequest(case, LNL))
    return pool


def serve_measure(ndatasets, rates, seconds, args=None, shapes=None):
    """The serving loop under Poisson arrivals at each of `rates` for
    `seconds` each, on `ndatasets` resident datasets of the serve
    workload's distribution, in the FP32 form and the plain FP64 form on
    the same arrivals.  Returns the per-rate p50/p99 and throughput of
    each precision, each precision's clocks, and the largest relative
    difference between the FP32 and FP64 lnLs of the same requests."""
    import numpy as np
    from crux_gb300 import _native, tune
    from crux_gb300.serve import LNL, MC3, PreparedRequest, Server
    t0 = time.perf_counter()
    base = make_serve_pool(ndatasets)
    # Each alignment is registered once as a resident dataset; requests
    # name it and carry only their tree and model.
    pool = [PreparedRequest(r.case, LNL, alignment=r.alignment,
                            dataset=i + 1) for i, r in enumerate(base)]
    mc3_pool = [PreparedRequest(r.case, MC3, mc3_gens=SERVE["mc3_gens"],
                                mc3_chains=2, seed=i + 1, session=i + 1,
                                alignment=r.alignment, dataset=i + 1)
                for i, r in enumerate(base) if r.alignment.ntaxa >= 4
                and r.case.pinv == 0.0]
    setup_s = time.perf_counter() - t0
    gpu = _native.load()
    # Tune the walker on the median-sized dataset of the pool.
    med = sorted(base, key=lambda r: r.req.ntaxa * r.req.npat)[len(base) // 2]
    out = {}
    for prec in ("fp32", "fp64"):
        if shapes and prec in shapes:
            sh = shapes[prec]
            tune.set_shape(gpu, sh["tile"], sh["tpp"], sh["ppt"], sh["budget"])
            out[prec + "_shape"] = dict(sh, lanes=1)
        else:
            lk = med.case.lik(lib=gpu, precision=prec, alignment=med.alignment)
            lk.prepare_plan()
            out[prec + "_shape"] = autotune(gpu, prec, args, lik=lk, lanes=False)
            del lk
        srv = Server(prec)
        for i, r in enumerate(base):
            srv.add_dataset(i + 1, r)
        # Warm: every dataset once (and each MC3 session created).
        for r in pool:
            srv.wait(srv.submit(r), timeout=600)
        for m in mc3_pool:
            srv.wait(srv.submit(m), timeout=600)
        per = []
        clocks = Clocks()
        clocks.start()
        for lam in rates:
            rng = np.random.default_rng(SERVE["seed"] + int(lam))
            n = max(10, int(lam * seconds))
            gaps = rng.exponential(1.0 / lam, n)
            kinds = rng.random(n) < SERVE["mc3_prob"]
            picks = rng.integers(len(pool), size=n)
            mpicks = rng.integers(len(mc3_pool), size=n)
            srv.reset_stats()
            tickets = []
            start = time.perf_counter()
            due = start
            for i in range(n):
                due += gaps[i]
                while True:
                    now = time.perf_counter()
                    if now >= due:
                        break
                    if due - now > 2e-4:
                        time.sleep(due - now - 1e-4)
                req = mc3_pool[mpicks[i]] if kinds[i] else pool[picks[i]]
                tickets.append((srv.submit(req), kinds[i], picks[i]))
            vals = []
            for t, is_mc3, pick in tickets:
                v, _ = srv.wait(t, timeout=600)
                if not is_mc3:
                    vals.append((pick, v))
            wall = time.perf_counter() - start
            st = srv.stats()
            per.append({"rate": lam, "requests": n, "p50_ms": st["p50_ms"],
                        "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                        "throughput_rps": n / wall,
                        "updates_per_s": st["updates"] / wall,
                        "max_batch": st["max_batch"], "batches": st["batches"],
                        "bytes_peak": st["bytes_peak"],
                        "deferrals": st["deferrals"]})
            out.setdefault(prec + "_vals", {}).update(dict(vals))
        out[prec + "_clocks"] = clocks.stop()
        srv.close()
        out[prec] = per
    errs = []
    for k, v in out["fp32_vals"].items():
        w = out["fp64_vals"].get(k)
        if w is not None:
            errs.append(abs(v - w) / abs(w))
    return {"workload": SERVE["workload"],
            "config": dict(SERVE, datasets=len(pool), rates=rates,
                           seconds_per_rate=seconds, setup_s=round(setup_s, 1)),
            "walker_shape": out["fp32_shape"],
            "walker_shape_fp64": out["fp64_shape"],
            "sweep_fp32": out["fp32"], "sweep_fp64": out["fp64"],
            "clocks": out["fp32_clocks"], "clocks_fp64": out["fp64_clocks"],
            "max_rel_err_fp32_vs_fp64": max(errs) if errs else None}


def run_serve(args, dist):
    """Serving loop under Poisson arrivals: p50/p99 latency and throughput
    of the FP32 form and of the plain FP64 form on the same arrivals."""
    rates = args.rates or SERVE["rates"]
    r = serve_measure(args.jobs or SERVE["datasets"], rates,
                      SERVE["seconds_per_rate"], args=args)
    best = max(r["sweep_fp32"], key=lambda x: x["throughput_rps"])
    line = {
        "metric": "serving: p50/p99 latency and throughput (FP32-scaled form)",
        "value": best["throughput_rps"], "unit": "requests/s",
        "n_gpus": 1, "steps": len(rates), "warmup": 1,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": r["config"], "walker_shape": r["walker_shape"],
        "walker_shape_fp64": r["walker_shape_fp64"],
        "sweep_fp32": r["sweep_fp32"], "sweep_fp64": r["sweep_fp64"],
        "clocks": r["clocks"], "clocks_fp64": r["clocks_fp64"],
        "max_rel_err_fp32_vs_fp64": r["max_rel_err_fp32_vs_fp64"],
    }
    print(json.dumps(line), flush=True)
    dist.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", type=lambda v: tuple(int(x) for x in v.split(",")),
                    default=None,
                    help="walker shape tile,threads_per_pattern,"
                         "patterns_per_thread,stack_bytes[,op_lanes] "
                         "instead of autotuning")
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU baseline and the oracle check")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="least CPU-baseline time for the default workload")
    ap.add_argument("--batch", type=int, default=256,
                    help="full-tree evaluations per step")
    ap.add_argument("--profile", action="store_true",
                    help="one plan (--precision) only, no e2e/CPU legs (for ncu)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"],
                    help="--profile: the plan's precision")
    ap.add_argument("--workload", default="tree128",
                    choices=["tree128", "batch256", "mc3", "mc3ref", "mc3small", "dirty64",
                             "compact",
                             "serve"])
    ap.add_argument("--rates", type=float, nargs="*", default=None,
                    help="serve: arrival rates (requests/s) to sweep")
    ap.add_argument("--gens", type=int, default=None,
                    help="mc3 workloads: generations to time")
    ap.add_argument("--chains", type=int, default=None,
                    help="MC3 workloads: number of chains")
    ap.add_argument("--jobs", type=int, default=None,
                    help="batch256: number of jobs (default 256)")
    ap.add_argument("--compact-shape", type=lambda v: [int(x) for x in v.split(",")],
                    default=None, help="compact: one ntaxa,nsites shape only")
    ap.add_argument("--batched-evals", type=int, default=32,
                    help="tree128: evaluations of the tree (each under its own "
                         "exchangeabilities) in the batched record (0: none)")
    ap.add_argument("--no-sub", action="store_true",
                    help="tree128: skip the MC3 and serving sub-records")
    ap.add_argument("--sub-mc3-gens", type=int, default=2000,
                    help="tree128: FP32 generations of the MC3 sub-record")
    ap.add_argument("--sub-mc3-gens64", type=int, default=500,
                    help="tree128: plain FP64 generations of the MC3 sub-record")
    ap.add_argument("--sub-serve-datasets", type=int, default=8,
                    help="tree128: resident datasets of the serving sub-record")
    ap.add_argument("--sub-serve-rates", type=float, nargs="*",
                    default=[100.0, 1000.0],
                    help="tree128: arrival rates of the serving sub-record")
    args = ap.parse_args()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    elif args.workload == "batch256":
        run_batch(args, dist)
    elif args.workload in MC3:
        run_mc3(args, dist)
    elif args.workload == "serve":
        run_serve(args, dist)
    elif args.workload == "dirty64":
        run_dirty(args, dist)
    elif args.workload == "compact":
        run_compact(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
