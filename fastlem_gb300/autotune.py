"""Schedule sweep: chooses the solve's launch shapes per size class on the GPU at hand.

    python -m fastlem_gb300.autotune [--out fastlem_gb300/schedule.json] [--quick]

For each size class -- single terrains of about 64k, 256k, 1M, 4M and 16M sites (the
16M benchmark terrain's generator at reduced scale: uniform sites, outlets on the left
and bottom borders, value-noise erodibility) and one packed batch of terrains of uneven
size -- it times generate() with set_max_iteration(8) (device time of the iteration
loop, after two warm-up solves) while varying, one knob at a time:
  kahn_min_width  where the Kahn rounds stop and the skeleton chain walks take over (the
                  round-versus-chain switch): the default rule n / 512 clamped to
                  [8192, 65536], times 1/16, 1/8, 1/4, 1/2 and 2;
  sized_grids     cooperative grids cut to the model's size, or the whole GPU;
  low_ilp         sites in flight per thread in the top-down Kahn rounds (1, 2, 4);
  walk_per_sm     chain walker blocks per SM (all that fit, 4, 2).
Each knob keeps the best value found before the next is tried.  The results go to a
JSON schedule (per class: the knobs, the time with the library defaults and with the
chosen knobs, every trial); the library's compiled-in schedule is set from it.  Every
shape gives the same bits (tests/test_gpu_tuning.py), so the sweep changes speed only.
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import _lib, workloads
from .api import TerrainGenerator, TerrainModel2D
from .batch import BatchGenerator

HERE = os.path.dirname(os.path.abspath(__file__))
SIZES = [65_536, 262_144, 1_048_576, 4_194_304, 16_000_000]


def _rule(n):
    return max(8192, min(65536, n // 512))


def _time_single(w, iters, reps):
    """Device ms per iteration of generate() on a fresh device model."""
    m = w.model
    fresh = TerrainModel2D(m.xs, m.ys, m.area, m.row_ptr, m.col, m.length, m.default_outlets)
    gen = TerrainGenerator.default().set_model(fresh).set_parameters(w.params).set_max_iteration(iters)
    for _ in range(2):
        gen.generate()
    best = math.inf
    for _ in range(reps):
        gen.generate()
        best = min(best, gen.last_loop_ms / max(1, gen.last_iterations))
    fresh.release()
    return best


def _time_packed(bw, iters, reps):
    bg = BatchGenerator().set_models(bw.models).set_parameters(bw.params).set_max_iteration(iters)
    for _ in range(2):
        bg.generate()
    best = math.inf
    for _ in range(reps):
        bg.generate()
        best = min(best, bg.last_loop_ms / max(1, bg.last_iterations))
    bg.batch.release()
    return best


def sweep(timer, n, log):
    """Coordinate sweep of the three knobs for one class; returns (default, best, trials)."""
    trials = []

    def run(width, ilp, walk, sized):
        old = _lib.set_tuning(kahn_min_width=width, low_ilp=ilp, walk_per_sm=walk,
                              sized_grids=sized)
        try:
            ms = timer()
        finally:
            _lib.set_tuning(**old)
        t = {"kahn_min_width": width, "low_ilp": ilp, "walk_per_sm": walk, "sized_grids": sized,
             "ms_per_iteration": ms}
        trials.append(t)
        log(f"  width {width:>7} ilp {ilp} walk/SM {walk} sized {sized}: {ms:.3f} ms/iteration")
        return ms

    rule = _rule(n)
    default = {"kahn_min_width": 0, "low_ilp": 4, "walk_per_sm": 0, "sized_grids": 0}
    default["ms_per_iteration"] = run(0, 4, 0, 0)
    best = dict(default)

    def knobs(**kw):
        d = {k: best[k] for k in ("kahn_min_width", "low_ilp", "walk_per_sm", "sized_grids")}
        d.update(kw)
        return d

    def tryit(**kw):
        k = knobs(**kw)
        ms = run(k["kahn_min_width"], k["low_ilp"], k["walk_per_sm"], k["sized_grids"])
        if ms < best["ms_per_iteration"]:
            best.update(k, ms_per_iteration=ms)

    for f in (0.0625, 0.125, 0.25, 0.5, 2.0):
        tryit(kahn_min_width=int(max(256, min(1 << 20, rule * f))))
    tryit(sized_grids=1)
    for ilp in (1, 2):
        tryit(low_ilp=ilp)
    for walk in (4, 2):
        tryit(walk_per_sm=walk)
    return default, best, trials


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "schedule.json"))
    ap.add_argument("--iters", type=int, default=8)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--quick", action="store_true", help="sizes up to 1M only")
    args = ap.parse_args()
    from . import build as fb
    fb.build()
    log = lambda s: print(s, flush=True)
    sizes = SIZES[:3] if args.quick else SIZES
    classes = []
    bounds = [int(math.sqrt(a * b)) for a, b in zip(sizes, sizes[1:])] + [0xFFFFFFFF]
    for n, bound in zip(sizes, bounds):
        t0 = time.time()
        w = workloads.sixteen_million(scale=n / 16_000_000)
        log(f"class <= {bound} sites: tuned on {w.model.num():,} sites (built in {time.time() - t0:.1f} s)")
        d, b, tr = sweep(lambda: _time_single(w, args.iters, args.reps), w.model.num(), log)
        classes.append({"max_sites": bound, "packed": False, "tuned_on_sites": w.model.num(),
                        "default": d, "best": b, "trials": tr})
        w.model.release()
    bw = workloads.batched(count=128)
    log(f"packed batches: tuned on {len(bw.models)} terrains, {bw.sites:,} sites")
    d, b, tr = sweep(lambda: _time_packed(bw, args.iters, args.reps), bw.sites, log)
    classes.append({"max_sites": 0xFFFFFFFF, "packed": True, "tuned_on_sites": bw.sites,
                    "tuned_on_terrains": len(bw.models), "default": d, "best": b, "trials": tr})
    out = {"what": "launch shapes per size class, chosen by fastlem_gb300/autotune.py",
           "metric": f"device ms per iteration of generate() with set_max_iteration({args.iters})",
           "device": _device_name(), "classes": classes}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    log("schedule written to " + args.out)
    for c in classes:
        s = c["best"]
        log(f"        {{{c['max_sites']:#x}u, {'true' if c['packed'] else 'false'}, "
            f"{{{s['low_ilp']}, {s['walk_per_sm']}, {s['kahn_min_width']}, "
            f"{'true' if s['sized_grids'] else 'false'}}}}},")


def _device_name():
    try:
        import subprocess
        r = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"],
                           capture_output=True, text=True, timeout=20)
        return r.stdout.strip().splitlines()[0]
    except Exception:
        return "unknown"


if __name__ == "__main__":
    main()
