"""Benchmark: fastlem generate() throughput (Msite-iters/s) on the 16M-site terrain.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one TerrainGenerator.generate() on the 16,000,000-site model with
set_max_iteration(M) (M = --iters, default 8): the first iteration routes the
initial-noise lakes, the rest are ordinary iterations.  Metric = sites x iterations
executed / time.
  value  device time of the iteration loop (CUDA events on the solver's stream), with
         the graph and parameters resident in HBM; inputs (1.6 GB) are larger than L2.
  e2e    the same work through the public API call with host arrays: parameter
         upload, initial elevations, the loop and the elevation download, host-timed.
Multi-GPU: a single terrain does not shard (replicas only); with N ranks each GPU
solves its own copy, value = all ranks' site-iterations / max rank time.
--impl reference times the CPU restatement of fastlem's own generate() (the oracle
port; fastlem is Rust and no Rust toolchain exists here) on the same model, one
bounded generate() per step, on rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msite-iters/s at 16M sites"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 10; 3 for the reference arm, whose steps take "
                         "seconds each)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="16m",
                    choices=["small", "1m", "16m", "batched", "served", "interp"])
    ap.add_argument("--interp-sites", type=int, default=1_000_000,
                    help="interp: sites of the terrain whose elevations are rendered")
    ap.add_argument("--interp-grid", type=int, default=4096,
                    help="interp: pixels per side of the rendering grid")
    ap.add_argument("--requests", type=int, default=64, help="served: requests in the stream")
    ap.add_argument("--slots", type=int, default=12, help="served: concurrent requests (worker threads)")
    ap.add_argument("--serve-iters", type=int, default=64,
                    help="served: set_max_iteration per request (fastlem's loop may not settle)")
    ap.add_argument("--terrains", type=int, default=512, help="batched: terrain count")
    ap.add_argument("--batch-iters", type=int, default=256,
                    help="batched: set_max_iteration per terrain (fastlem's loop may not settle)")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--iters", type=int, default=8, help="set_max_iteration per step")
    ap.add_argument("--cpu-iters", type=int, default=1, help="iterations in the CPU sample")
    ap.add_argument("--cpu-threads", type=int, default=0,
                    help="reference arm: replica threads (0: every core the memory allows)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="16M run: skip the batched (C4) and served (C5) summaries")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 3 if args.impl == "reference" else 10
    return args


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 100 ms.  The sampler is started
    (and its first sample awaited, so that nvidia-smi's start-up does not fall into the
    timed region) before timing begins; summary() keeps the samples taken inside the
    timed region (start() .. stop())."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpus):
        self.gpus = gpus
        self.proc = None
        self.lines = []                 # (arrival time, line)
        self.t0 = self.t1 = None
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=15)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))
            self.first.set()

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self):
        self.t1 = time.perf_counter()
        if self.proc:                   # one more sample covers the region's end
            deadline = self.t1 + 0.3
            while time.perf_counter() < deadline and not any(t >= self.t1 for t, _ in self.lines):
                time.sleep(0.02)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.t0 is not None and self.t1 is not None:
            # samples taken in the region, plus the first one after it (it covers the
            # region's last 100 ms)
            inside = [(t, ln) for t, ln in lines if self.t0 <= t <= self.t1]
            after = [(t, ln) for t, ln in lines if t > self.t1][:max(1, self.gpus)]
            lines = inside + after
        for _, ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) >= self.gpus:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (read + write) of one launch from an ncu capture, per unit the kernel
# processes; a capture of the full 16M workload does not fit the profiling size rule,
# so the 1M config's launch (8th iteration of a generate(), --set full) is scaled by
# the units (traffic grows with them).
NCU_TRAFFIC = {
    # 56.76 MB over the 939,485 Kahn-region sites (1,000,000 - 60,515 skeleton sites)
    "kahn_rounds": (56.763e6 / 939_485, "kahn_sites",
                    "ncu dram__bytes_read+write of one k_kahn launch on the 1M config "
                    "(8th iteration), scaled by Kahn-region sites"),
    # 3.064 MB over 60,515 skeleton sites
    "skeleton_up": (3.064e6 / 60_515, "skeleton_sites",
                    "ncu dram__bytes_read+write of one k_s_bottom_up launch on the 1M config "
                    "(8th iteration), scaled by skeleton sites"),
    # 113.38 MB over 1,000,000 sites
    "receivers": (113.38e6 / 1_000_000, "sites",
                  "ncu dram__bytes_read+write of one k_receivers launch on the 1M config "
                  "(8th iteration), scaled by sites"),
    # 52.40 MB over the 939,485 Kahn-region sites
    "rounds_down": (52.40e6 / 939_485, "kahn_sites",
                    "ncu dram__bytes_read+write of one k_low_top_down launch on the 1M config "
                    "(8th iteration), scaled by Kahn-region sites"),
    # 39.41 MB over 1,000,000 sites
    "response_w": (39.41e6 / 1_000_000, "sites",
                   "ncu dram__bytes_read+write of one k_w launch on the 1M config "
                   "(8th iteration), scaled by sites"),
}


def measured_traffic(kernel, basin, n):
    if kernel not in NCU_TRAFFIC:
        return None, "no ncu capture for this kernel"
    per, unit, src = NCU_TRAFFIC[kernel]
    units = {"skeleton_sites": basin["skeleton_sites"], "sites": n,
             "kahn_sites": n - basin["skeleton_sites"]}[unit]
    return per * units, src


def make_workload(args):
    from fastlem_gb300 import workloads
    t = time.time()
    w = workloads.CONFIGS[args.config](args.scale)
    return w, time.time() - t


def run_cpu_sample(w, iters):
    """The oracle (CPU restatement of fastlem's generate) on this model, bounded to
    `iters` iterations; returns (site-iterations per second, iterations, seconds,
    elevations)."""
    from oracle import oracle as orc
    from tests import graphs
    p = w.params
    r = orc.generate(graphs.from_model(w.model), p.base, p.erodibility, p.uplift, p.is_outlet,
                     max_slope=p.max_slope, max_iter=iters)
    return w.model.num() * r["iters"] / r["seconds"], r["iters"], r["seconds"], r["elev"]


def gpu_matches_cpu_sample(w, iters, want_iters, want_elev):
    """The GPU's generate() with the CPU sample's iteration bound, compared bit for bit
    with the sample's elevations (the measured CPU work is the same solve)."""
    from fastlem_gb300 import TerrainGenerator
    gen = (TerrainGenerator.default().set_model(w.model).set_parameters(w.params)
           .set_max_iteration(iters))
    got = gen.generate().elevations()
    same = (gen.last_iterations == want_iters and
            np.array_equal(np.ascontiguousarray(got).view(np.uint64),
                           np.ascontiguousarray(want_elev).view(np.uint64)))
    return {"iterations": int(want_iters), "bit_exact": bool(same)}


def cold_call(w, iters):
    """What a drop-in generate() pays when it builds its model each call: a fresh
    device graph (Hilbert order, CSR relabelling, upload) and a first generate() that
    also computes the lake order, from pageable host arrays, host-timed."""
    from fastlem_gb300 import TerrainGenerator
    from fastlem_gb300.api import TerrainModel2D
    m = w.model
    fresh = TerrainModel2D(m.xs, m.ys, m.area, m.row_ptr, m.col, m.length, m.default_outlets)
    t0 = time.perf_counter()
    fresh.handle()
    t1 = time.perf_counter()
    gen = TerrainGenerator.default().set_model(fresh).set_parameters(w.params).set_max_iteration(iters)
    gen.generate()
    t2 = time.perf_counter()
    from fastlem_gb300 import _lib
    rank_ms, rank_where = _lib.rank_info(fresh.handle())
    fresh.release()
    return {"graph_create_s": t1 - t0, "first_generate_s": t2 - t1, "total_s": t2 - t0,
            "iterations": gen.last_iterations,
            "lake_order": {"ms": rank_ms, "computed_on": rank_where},
            "what": "fl_graph_create + first fl_generate (lake order included), pageable "
                    "host arrays, host wall clock"}


def cpu_pool_sample(models, params, iters, per_terrain_iters, budget_s=12.0):
    """All host cores on independent terrains: the oracle in a thread pool (its C calls
    release the GIL), on terrains spread over the workload's sizes (every k-th by size),
    each bounded to min(iters, what one core does in about budget_s).  Returns
    (aggregate site-iterations per second, threads, description); the workload's
    terrains/s on the host is that rate over `per_terrain_iters` (the mean
    site-iterations of one of its terrains, from the GPU run)."""
    import concurrent.futures as cf
    import threading
    from oracle import oracle as orc
    from tests import graphs
    threads = os.cpu_count() or 1
    order = np.argsort([m.num() for m in models], kind="stable")
    k = min(len(order), 4 * threads)
    pick = order[np.linspace(0, len(order) - 1, k).round().astype(int)]
    per_core = 0.6e6 * budget_s                          # site-iterations a core does
    done = []
    lock = threading.Lock()

    def one(i):
        m, p = models[i], params[i]
        mi = int(max(1, min(iters, per_core // m.num())))
        r = orc.generate(graphs.from_model(m), p.base, p.erodibility, p.uplift, p.is_outlet,
                         max_slope=p.max_slope, max_iter=mi)
        with lock:
            done.append(m.num() * r["iters"])

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, pick))
    secs = time.perf_counter() - t0
    rate = sum(done) / secs
    desc = (f"oracle generate() on {len(pick)} of the {len(models)} terrains (every k-th by "
            f"size, {min(m.num() for m in models):,}-{max(m.num() for m in models):,} sites), "
            f"each bounded to <= {iters} iterations and ~{int(per_core):,} site-iterations, "
            f"{threads} threads, {secs:.1f} s; terrains/s = site-iterations/s over the mean "
            f"{per_terrain_iters:,.0f} site-iterations of a terrain in the GPU run")
    return rate, threads, desc


def workload_name(w):
    c = w.config
    return (f"{w.name}: {c['sites']:,} sites uniform in [0,{c['box']:g}]^2 seed {c['seed']}, "
            f"relax {c['relax']}, outlets {c['outlets']}, erodibility {c['erodibility']}")


def host_replica_threads(n):
    """Replica threads the host can run for an n-site model: every core, bounded by the
    available memory (about 250 B per site for one oracle solve's state)."""
    cores = os.cpu_count() or 1
    try:
        with open("/proc/meminfo") as f:
            avail = next(int(l.split()[1]) * 1024 for l in f if l.startswith("MemAvailable:"))
    except (OSError, StopIteration, ValueError):
        return 1
    return max(1, min(cores, int(avail * 0.6 // (250 * max(1, n)))))


def bench_reference(args, d):
    """The reference's path on the host cores: fastlem's generate() is single-threaded,
    so all cores run independent replicas of the same solve (one per thread; the
    oracle's C calls release the GIL), each bounded to --cpu-iters iterations per step.
    value = site-iterations of all replicas / wall time of the step."""
    if d.rank != 0:
        return
    import concurrent.futures as cf
    from oracle import build as ob
    from oracle import oracle as orc
    from tests import graphs
    ob.build()
    orc.lib()
    w, build_s = make_workload(args)
    n = w.model.num()
    g = graphs.from_model(w.model)
    p = w.params
    threads = args.cpu_threads or host_replica_threads(n)

    def solve(_):
        r = orc.generate(g, p.base, p.erodibility, p.uplift, p.is_outlet,
                         max_slope=p.max_slope, max_iter=args.cpu_iters)
        return r["iters"]

    secs, its = 0.0, 0
    with cf.ThreadPoolExecutor(threads) as ex:
        for _ in range(args.warmup):
            list(ex.map(solve, range(threads)))
        for _ in range(args.steps):
            t0 = time.perf_counter()
            its += sum(ex.map(solve, range(threads)))
            secs += time.perf_counter() - t0
    value = n * its / secs / 1e6
    sample = (f"{threads} concurrent replicas (one thread each) of generate() with "
              f"set_max_iteration({args.cpu_iters}) on the same {n:,}-site model per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Msite-iters/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(w), "iterations_per_step": args.cpu_iters,
                   "host_threads": threads, "host_cores": os.cpu_count()},
        "cpu_baseline": {"value": value, "unit": "Msite-iters/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Msite-iters/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_gpu(args, d):
    from fastlem_gb300 import TerrainGenerator, build as fb
    from fastlem_gb300 import _lib
    fb.build()
    L = _lib.lib()
    _lib.check(L.fl_select_device(d.local))
    w, build_s = make_workload(args)
    m, p = w.model, w.params
    n = m.num()
    h = m.handle()
    # host arrays in page-locked memory: each step uploads them and downloads the
    # elevations by DMA
    pp = p.pinned()
    out = _lib.pinned_empty(n, np.float64)
    gen = TerrainGenerator.default().set_model(m).set_parameters(pp).set_max_iteration(args.iters)

    for _ in range(args.warmup):
        gen.generate(out=out)

    # timed region: K steps, per-kernel CUDA-event timing on the solver stream
    L.fl_graph_reset_stats(h)
    _lib.check(L.fl_graph_set_timing(h, 1))
    loop_ms, total_ms, iters = 0.0, 0.0, 0
    with ClockSampler(max(1, args.gpus)) as clocks:
        d.barrier()
        clocks.start()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            gen.generate(out=out)
            loop_ms += gen.last_loop_ms
            total_ms += gen.last_total_ms
            iters += gen.last_iterations
        wall_ms = 1000 * (time.perf_counter() - t0)
        clocks.stop()
        d.barrier()
    _lib.check(L.fl_graph_set_timing(h, 0))
    stats = _lib.kernel_stats(h)
    basin = _lib.basin_stats(h)

    site_iters = d.sum(n * iters)
    loop_max = d.max(loop_ms)
    total_max = d.max(total_ms)
    value = site_iters / (loop_max / 1000) / 1e6
    e2e = site_iters / (total_max / 1000) / 1e6
    launches = int(sum(v[0] for v in stats.values()))
    if d.rank != 0:
        return

    # dominant kernel class by device time
    dom = max(stats.items(), key=lambda kv: kv[1][1])
    dname, (dl, dms, dbytes) = dom
    peak, peak_kind = peak_hbm()
    achieved = (dbytes / dl) / ((dms / dl) / 1000) / 1e9 if dl and dms else 0.0
    all_bytes = sum(v[2] for v in stats.values())
    all_ms = sum(v[1] for v in stats.values())
    traffic, traffic_src = measured_traffic(dname, basin, n)
    # the whole solve against the per-site-iteration byte count of the path: per-site
    # inputs 37 B, 12 B per slot, intermediates 48 B, output 8 B
    dbar = float(m.row_ptr[-1]) / n
    b_alg = 93.0 + 12.0 * dbar
    whole = b_alg * site_iters / (loop_max / 1000) / 1e9
    roof = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "traffic_source": traffic_src,
            "bytes_per_launch": dbytes / max(1, dl), "ms_per_launch": dms / max(1, dl),
            "launches": dl,
            # every kernel class together: algorithmic bytes of the whole solve over its
            # device time
            "all_kernels": {"achieved": all_bytes / (all_ms / 1000) / 1e9 if all_ms else 0.0,
                            "frac": (all_bytes / (all_ms / 1000) / 1e9 / peak) if all_ms else 0.0,
                            "bytes_per_iteration": all_bytes / max(1, iters)},
            # (93 + 12 d) B per site-iteration over the loop's device time
            "whole_solve": {"bytes_per_site_iteration": b_alg, "mean_degree": dbar,
                            "achieved": whole, "frac": whole / peak}}
    share = {k: round(v[1] / max(1e-9, sum(x[1] for x in stats.values())), 4)
             for k, v in stats.items() if v[0]}
    # loop time on the device not covered by any launch group: launch latency and the
    # host round trips of the iteration loop
    idle = {"ms_per_step": (loop_ms - all_ms) / args.steps,
            "frac": (loop_ms - all_ms) / loop_ms if loop_ms else 0.0,
            "host_syncs_per_iteration": _lib.host_syncs(h) / max(1, iters)}
    cpu = None
    if not args.no_cpu_baseline and args.gpus == 1:
        from oracle import build as ob
        ob.build()
        v, it, s, elev = run_cpu_sample(w, args.cpu_iters)
        cpu = {"value": v / 1e6, "unit": "Msite-iters/s", "cores": 1, "kind": "port",
               "sample": f"oracle generate() with set_max_iteration({it}) on the same {n:,}-site "
                         f"model, {s:.1f} s, 1 thread", "host_cores": os.cpu_count(),
               "gpu_parity": gpu_matches_cpu_sample(w, args.cpu_iters, it, elev),
               "parity_note": "GPU results equal the oracle bit for bit; the oracle restates "
                              "fastlem's generate() and is not pinned against fastlem's own "
                              "binary (no Rust toolchain, no reference goldens)"}
        del elev
    # base, erodibility, uplift, is_outlet (+ max_slope when given), from pinned memory
    h2d = n * (8 + 8 + 8 + 1) + (n * 8 if p.max_slope is not None else 0)
    d2h = n * 8
    line = {
        "metric": METRIC, "value": value, "unit": "Msite-iters/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": loop_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_name(w), "iterations_per_step": args.iters,
                   "site_iterations_per_step": n * iters // max(1, args.steps),
                   "parallelism": f"replicas x{args.gpus}",
                   "l2": "inputs larger than L2 (CSR and per-site arrays ~1.6 GB)",
                   "graph_build_s": round(build_s, 1)},
        "e2e": {"value": e2e, "unit": "Msite-iters/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "host_buffers": "page-locked (fl_host_alloc)"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "kernel_time_share": share,
        "idle_gap": idle,
        "basin_last_iteration": basin,
        "clocks": clocks.summary(),
        "wall_ms_timed": wall_ms,
    }
    if args.gpus == 1:
        line["cold_call"] = cold_call(w, args.iters)
    if not args.no_extras and args.gpus == 1 and args.config == "16m":
        # the other two parts of the headline metric, on the same GPU after the 16M run
        import copy
        ea = copy.copy(args)
        ea.steps, ea.warmup, ea.batch_iters, ea.requests, ea.serve_iters = 2, 1, 64, 32, 64
        b = bench_batched(ea, d, emit=False)
        line["batched"] = {k: b[k] for k in ("metric", "value", "unit", "e2e", "plain_loop",
                                              "speedup_vs_plain_loop", "identical_to_plain",
                                              "cpu_baseline")}
        line["batched"]["config"] = b["config"]
        sv = bench_served(ea, d, emit=False)
        line["served"] = {k: sv[k] for k in ("metric", "value", "unit", "latency_ms",
                                              "sequential_plain", "speedup_vs_sequential",
                                              "identical_to_plain", "cpu_baseline", "server",
                                              "mean_in_service", "queue_ms")}
        line["served"]["config"] = sv["config"]
        it = bench_interp(ea, d, emit=False)
        line["interp"] = {k: it[k] for k in ("metric", "value", "unit", "e2e", "cpu_baseline",
                                             "identical_to_host", "config")}
    print(json.dumps(line), flush=True)


def bench_batched(args, d, emit=True):
    """C4: 512 terrains of uneven size solved as one packed graph, against the plain
    per-terrain loop (one TerrainGenerator.generate() after another) on the same GPU.
    A step solves every terrain to convergence (generator defaults)."""
    from fastlem_gb300 import TerrainGenerator, build as fb, workloads
    from fastlem_gb300.batch import BatchGenerator
    fb.build()
    from fastlem_gb300 import _lib
    _lib.check(_lib.lib().fl_select_device(d.local))
    t0 = time.time()
    w = workloads.batched(count=args.terrains)
    build_s = time.time() - t0
    count, sites = len(w.models), w.sites
    bg = (BatchGenerator().set_models(w.models).set_parameters(w.params)
          .set_max_iteration(args.batch_iters))
    gens = [TerrainGenerator.default().set_model(m).set_parameters(p)
            .set_max_iteration(args.batch_iters) for m, p in zip(w.models, w.params)]
    # warm-up: resident graphs, lake ranks, caches
    for _ in range(max(1, args.warmup)):
        got = bg.generate()
    for g in gens:
        g.generate()
    # plain per-terrain loop: one pass, device loop time and wall time
    d.barrier()
    plain_loop_ms, plain_iters = 0.0, 0
    t = time.perf_counter()
    plain = []
    for g in gens:
        plain.append(g.generate().elevations())
        plain_loop_ms += g.last_loop_ms
        plain_iters += g.last_iterations
    plain_wall = time.perf_counter() - t
    identical = all(np.array_equal(a.view(np.uint64), b.elevations().view(np.uint64))
                    for a, b in zip(plain, got))
    # batched: K steps
    loop_ms, total_ms = 0.0, 0.0
    with ClockSampler(max(1, args.gpus)) as clocks:
        d.barrier()
        clocks.start()
        t = time.perf_counter()
        for _ in range(args.steps):
            bg.generate()
            loop_ms += bg.last_loop_ms
            total_ms += bg.last_total_ms
        wall = time.perf_counter() - t
        clocks.stop()
        d.barrier()
    loop_max = d.max(loop_ms)
    total_max = d.max(total_ms)
    if d.rank != 0:
        return
    t_iters = np.asarray(bg.last_terrain_iterations, np.int64)
    site_iters = int(sum(m.num() * int(i) for m, i in zip(w.models, t_iters)))
    value = count * args.steps * d.world / (loop_max / 1000)
    e2e = count * args.steps * d.world / (total_max / 1000)
    plain_tps = count / (plain_loop_ms / 1000)
    plain_tps_wall = count / plain_wall
    h2d = sites * (8 + 8 + 8 + 1)
    cpu = None
    if not args.no_cpu_baseline and args.gpus == 1:
        try:
            rate, thr, desc = cpu_pool_sample(w.models, w.params, args.batch_iters,
                                              site_iters / count)
            cpu = {"value": rate / (site_iters / count), "unit": "terrains/s", "cores": thr,
                   "kind": "port", "site_iterations_per_s": rate, "sample": desc}
        except Exception as e:   # the GPU figures stand without it
            cpu = {"unavailable": f"{type(e).__name__}: {e}"}
    line = {
        "metric": "batched terrains/s (512 terrains, 4,096-262,144 sites)",
        "value": value, "unit": "terrains/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": loop_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"batched: {count} terrains, {sites:,} sites, n log-uniform "
                               f"[4096, 262144] seed 3, border outlets 2%, lognormal(0,0.5) "
                               f"erodibility, until an iteration changes nothing or "
                               f"{args.batch_iters} iterations",
                   "terrains_at_iteration_cap": int((t_iters >= args.batch_iters).sum()),
                   "packed_iterations": bg.last_iterations,
                   "terrain_iterations": {"min": int(t_iters.min()), "median": float(np.median(t_iters)),
                                          "max": int(t_iters.max())},
                   "site_iterations_per_step": site_iters, "graph_build_s": round(build_s, 1),
                   "parallelism": f"replicas x{args.gpus}"},
        "e2e": {"value": e2e, "unit": "terrains/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": sites * 8},
        "plain_loop": {"terrains_per_s": plain_tps, "terrains_per_s_wall": plain_tps_wall,
                       "loop_ms": plain_loop_ms, "wall_s": plain_wall,
                       "site_iterations": int(sum(m.num() * g.last_iterations
                                                  for m, g in zip(w.models, gens)))},
        "speedup_vs_plain_loop": value / plain_tps,
        "speedup_vs_plain_loop_wall": (count * args.steps / wall) / plain_tps_wall,
        "identical_to_plain": identical,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def bench_served(args, d, emit=True):
    """C5: a Poisson stream of generate() requests (200 req/s, 16,384-4,194,304 sites)
    replayed in real time, once through the server (concurrent requests, resident
    models, 120 GB HBM admission budget) and once one request at a time through the
    plain path; latency = completion - arrival.  Both start cold (each request's graph
    is uploaded by its first solve)."""
    from fastlem_gb300 import TerrainGenerator, build as fb, workloads
    from fastlem_gb300.serve import TerrainServer
    fb.build()
    from fastlem_gb300 import _lib
    _lib.check(_lib.lib().fl_select_device(d.local))
    t0 = time.time()
    w = workloads.served(count=args.requests)
    build_s = time.time() - t0
    R = len(w.models)
    cap = args.serve_iters
    # CUDA context and library warm-up on a throw-away model
    tiny = workloads.small(scale=0.1)
    TerrainGenerator.default().set_model(tiny.model).set_parameters(tiny.params).generate()

    def replay(start_one, finish_all):
        t0 = time.perf_counter()
        handles = []
        for i in range(R):
            now = time.perf_counter() - t0
            if now < w.arrivals[i]:
                time.sleep(w.arrivals[i] - now)
            handles.append(start_one(i, t0))
        res = finish_all(handles, t0)
        return res, time.perf_counter() - t0

    # sequential plain GPU path
    gens = [TerrainGenerator.default().set_model(m).set_parameters(p).set_max_iteration(cap)
            for m, p in zip(w.models, w.params)]
    def seq_one(i, t0):
        e = gens[i].generate().elevations()
        return e, (time.perf_counter() - t0 - w.arrivals[i]) * 1000, gens[i].last_iterations
    seq, seq_span = replay(seq_one, lambda hs, t0: hs)
    # served
    with ClockSampler(max(1, args.gpus)) as clocks:
        with TerrainServer(hbm_budget_bytes=120 * 10**9, slots=args.slots) as srv:
            ids = [srv.add_model(m) for m in w.models]
            clocks.start()
            served, span = replay(lambda i, t0: srv.submit(ids[i], w.params[i], cap),
                                  lambda hs, t0: [srv.wait(h) for h in hs])
            clocks.stop()
            stats = srv.stats()
    if d.rank != 0:
        return
    lat = np.array([info["latency_ms"] for _, info in served])
    seq_lat = np.array([l for _, l, _ in seq])
    identical = all(np.array_equal(a.view(np.uint64), t.elevations().view(np.uint64))
                    for (a, _, _), (t, _) in zip(seq, served))
    iters = np.array([info["iterations"] for _, info in served])
    site_iters = int(sum(m.num() * int(i) for m, i in zip(w.models, iters)))
    value = R / span
    cpu = None
    if not args.no_cpu_baseline and args.gpus == 1:
        try:
            rate, thr, desc = cpu_pool_sample(w.models, w.params, cap, site_iters / R)
            cpu = {"value": rate / (site_iters / R), "unit": "terrains/s", "cores": thr,
                   "kind": "port", "site_iterations_per_s": rate, "sample": desc}
        except Exception as e:   # the GPU figures stand without it
            cpu = {"unavailable": f"{type(e).__name__}: {e}"}
    line = {
        "metric": "served terrains/s and p99 latency (Poisson 200 req/s, 16,384-4,194,304 sites)",
        "value": value, "unit": "terrains/s", "n_gpus": args.gpus, "steps": 1, "warmup": 1,
        "ms_per_step": span * 1000, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"served: {R} requests, Poisson {w.config['rate_per_s']:g}/s seed 5, "
                               f"n log-uniform [16384, 4194304], {w.config['sites']:,} sites, "
                               f"per-request erodibility field, border outlets 2%, until an "
                               f"iteration changes nothing or {cap} iterations",
                   "slots": args.slots, "hbm_budget_gb": 120,
                   "requests_at_iteration_cap": int((iters >= cap).sum()),
                   "site_iterations": site_iters, "graph_build_s": round(build_s, 1)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max())},
        "e2e": {"value": value, "unit": "terrains/s",
                "h2d_bytes_per_step": int(sum(m.num() * 25 for m in w.models)),
                "d2h_bytes_per_step": int(sum(m.num() * 8 for m in w.models))},
        "sequential_plain": {"terrains_per_s": R / seq_span,
                             "latency_ms": {"p50": float(np.percentile(seq_lat, 50)),
                                            "p99": float(np.percentile(seq_lat, 99))}},
        "speedup_vs_sequential": (R / span) / (R / seq_span),
        "identical_to_plain": identical,
        "cpu_baseline": cpu,
        "server": stats,
        # mean requests in service over the span (solve time of all requests / span)
        "mean_in_service": float(sum(info["solve_ms"] for _, info in served) / (span * 1000)),
        "queue_ms": {"p50": float(np.percentile([i["queue_ms"] for _, i in served], 50)),
                     "max": float(max(i["queue_ms"] for _, i in served))},
        "clocks": clocks.summary(),
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def bench_interp(args, d, emit=True):
    """Terrain2D::get_elevation over a rendering grid (src/models/surface/terrain.rs:35-38,
    the per-pixel loop of examples/landscape_evolution.rs at a larger size): a terrain of
    random sites in [0,4000]^2 rendered on an n x n pixel grid covering the box.  value:
    device-resident queries (fl_interpolate_device); e2e: host arrays in and out
    (fl_interpolate_gpu); cpu_baseline: the host fl_interpolate on every core, on a band
    of rows; identical_to_host: the two give the same bits on that band."""
    import torch
    from fastlem_gb300 import Site2D, TerrainModel2DBulider, build as fb
    from fastlem_gb300 import _lib
    from fastlem_gb300.api import TerrainInterpolator2D
    fb.build()
    _lib.check(_lib.lib().fl_select_device(d.local))
    torch.cuda.set_device(d.local)
    t0 = time.time()
    model = TerrainModel2DBulider.from_random_sites(
        args.interp_sites, Site2D(0.0, 0.0), Site2D(4000.0, 4000.0), seed=7).build()
    elev = np.random.default_rng(7).uniform(0.0, 500.0, model.num())
    it = TerrainInterpolator2D(model.xs, model.ys)
    build_s = time.time() - t0
    g = args.interp_grid
    px = (np.arange(g, dtype=np.float64) + 0.5) * (4000.0 / g)
    QX, QY = np.meshgrid(px, px)
    qx, qy = np.ascontiguousarray(QX.ravel()), np.ascontiguousarray(QY.ravel())
    count = qx.size
    dev = torch.device("cuda", d.local)
    tf, tx, ty = (torch.from_numpy(a).to(dev) for a in (elev, qx, qy))
    out = torch.empty(count, dtype=torch.float64, device=dev)
    found = torch.empty(count, dtype=torch.uint8, device=dev)
    for _ in range(max(3, args.warmup)):
        it.interpolate_device(tf, tx, ty, out, found)
    steps = max(1, args.steps)
    torch.cuda.synchronize()
    d.barrier()
    t = time.perf_counter()
    for _ in range(steps):
        it.interpolate_device(tf, tx, ty, out, found)
    dev_s = (time.perf_counter() - t) / steps
    host_out = _lib.pinned_empty(count, np.float64)
    hx, hy = _lib.pinned_empty(count, np.float64), _lib.pinned_empty(count, np.float64)
    hx[:], hy[:] = qx, qy
    for _ in range(2):
        v, ok = it.interpolate_many(elev, hx, hy, gpu=True)
    t = time.perf_counter()
    for _ in range(steps):
        v, ok = it.interpolate_many(elev, hx, hy, gpu=True)
    e2e_s = (time.perf_counter() - t) / steps
    dev_vals = out.cpu().numpy()
    # host baseline on a band of rows (8M queries: about a second on 16 host threads)
    rows = max(1, min(g, int(8_000_000 // g)))
    band = slice(((g - rows) // 2) * g, ((g - rows) // 2 + rows) * g)
    it.interpolate_many(elev, qx[:1000], qy[:1000])
    t = time.perf_counter()
    hv, hok = it.interpolate_many(elev, qx[band], qy[band])
    cpu_s = time.perf_counter() - t
    same = bool(np.array_equal(hv.view(np.uint64), dev_vals[band].view(np.uint64)) and
                np.array_equal(hok, found.cpu().numpy()[band].astype(bool)) and
                np.array_equal(v.view(np.uint64), dev_vals.view(np.uint64)))
    cores = min(16, os.cpu_count() or 1)
    line = {
        "metric": f"natural-neighbour queries/s ({g}x{g} rendering grid, {model.num():,} sites)",
        "value": count / dev_s / 1e6, "unit": "Mqueries/s", "n_gpus": 1,
        "e2e": {"value": count / e2e_s / 1e6, "unit": "Mqueries/s",
                "h2d_bytes_per_step": 16 * count + 8 * model.num(),
                "d2h_bytes_per_step": 9 * count},
        "cpu_baseline": {"value": (band.stop - band.start) / cpu_s / 1e6, "unit": "Mqueries/s",
                         "cores": cores, "kind": "port",
                         "sample": f"host fl_interpolate (the same construction on host threads) on "
                                   f"{rows} middle rows of the grid ({band.stop - band.start:,} "
                                   f"queries), {cpu_s:.2f} s"},
        "identical_to_host": same,
        "ms_per_step": dev_s * 1000, "e2e_ms_per_step": e2e_s * 1000,
        "found_fraction": float(found.float().mean().item()),
        "config": {"workload": f"interp: {model.num():,} random sites in [0,4000]^2 seed 7 "
                               f"(from_random_sites), uniform(0,500) elevations, {g}x{g} pixel "
                               f"centres", "queries_per_step": count, "steps": steps,
                   "model_and_triangulation_build_s": round(build_s, 1)},
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def main():
    args = parse()
    d = Dist()
    if args.config == "batched" and args.impl != "reference":
        bench_batched(args, d)
        return
    if args.config == "served" and args.impl != "reference":
        bench_served(args, d)
        return
    if args.config == "interp" and args.impl != "reference":
        bench_interp(args, d)
        return
    if args.impl == "reference":
        bench_reference(args, d)
    else:
        bench_gpu(args, d)


if __name__ == "__main__":
    main()
