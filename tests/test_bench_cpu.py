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
