"""bench.py's host-side baselines, on the CPU: the all-cores sample over independent
terrains (the batched and served lines' cpu_baseline) and the reference arm's replica
thread count."""
import os

import numpy as np

import bench
from fastlem_gb300 import workloads


def test_all_cores_sample_over_terrains():
    w = workloads.batched(count=6, lo=4096, hi=8192, seed=1)
    rate, threads, desc = bench.cpu_pool_sample(w.models, w.params, 4, per_terrain_iters=20000.0,
                                                budget_s=1.0)
    assert rate > 0 and np.isfinite(rate)
    assert 1 <= threads <= (os.cpu_count() or 1)
    assert "terrains" in desc and f"{threads} threads" in desc


def test_replica_threads_fit_memory():
    t = bench.host_replica_threads(16_000_000)
    assert 1 <= t <= (os.cpu_count() or 1)
    assert bench.host_replica_threads(1000) == (os.cpu_count() or 1)


def test_clock_summary_keeps_the_timed_region():
    """Samples before the timed region (nvidia-smi's start-up) are dropped; the first one
    after it is kept (it covers the region's last interval); throttle reasons are read
    from the kept samples only."""
    c = bench.ClockSampler(1)
    row = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, Not Active"
    c.lines = [(0.5, row.format(sm=990, hw="Active")),      # before the region
               (1.2, row.format(sm=2070, hw="Not Active")),
               (1.3, row.format(sm=2065, hw="Not Active")),
               (2.05, row.format(sm=2070, hw="Not Active")),  # first after the region
               (2.5, row.format(sm=1000, hw="Active"))]
    c.t0, c.t1 = 1.0, 2.0
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["reasons"] == []
    c.t0 = c.t1 = None                                       # no region: every sample
    assert c.summary()["samples"] == 5 and "hw_slowdown" in c.summary()["reasons"]
