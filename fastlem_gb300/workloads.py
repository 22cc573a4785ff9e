"""Seeded synthetic workloads (sites, graph, parameters) for the solve.

No public dataset is involved; every config is generated here from a seed:
  small   10,000 sites in [0,100]^2, seed 42, one Lloyd relaxation, outlets within 2.0 of
          the border, erodibility 1.0, generator defaults (the reference's CPU case).
  1m      1,000,000 sites in [0,1000]^2, seed 7, one Lloyd relaxation, outlets within 5.0
          of the border, erodibility clamp(exp(N(0,0.5)) * (0.5 + V), 0.1, 4.0) with V a
          4-octave value-noise field in [0,1).
  16m     16,000,000 sites in [0,4000]^2, seed 11, no relaxation, outlets only within 5.0
          of the left and bottom borders, erodibility 1 + 0.8 * (2V - 1).
Sites are drawn like fastlem's `from_random_sites` (x then y per site with gen_range)
from StdRng::seed_from_u64(seed).  `scale` shrinks a config's site count and box side
together (same density) for parity runs at reduced size.
"""
import math
import os
from dataclasses import dataclass, field

import numpy as np

from .api import ParameterArrays, Site2D, TerrainModel2DBulider


def _hash01(ix, iy, octave, seed):
    """Uniform [0,1) lattice values from a 64-bit integer hash (splitmix64 finaliser)."""
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
             ^ iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)
             ^ np.uint64((octave * 0x165667B19E3779F9 + seed * 0xD6E8FEB86659FD93) & 0xFFFFFFFFFFFFFFFF))
        h ^= h >> np.uint64(30)
        h *= np.uint64(0xBF58476D1CE4E5B9)
        h ^= h >> np.uint64(27)
        h *= np.uint64(0x94D049BB133111EB)
        h ^= h >> np.uint64(31)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def value_noise(x, y, seed, wavelength, octaves=4, persistence=0.5):
    """Smooth value noise in [0,1): lattice spacing `wavelength`, halved per octave."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    total = np.zeros_like(x)
    amp, norm, wl = 1.0, 0.0, float(wavelength)
    for o in range(octaves):
        gx, gy = x / wl, y / wl
        ix, iy = np.floor(gx), np.floor(gy)
        fx, fy = gx - ix, gy - iy
        sx, sy = fx * fx * (3 - 2 * fx), fy * fy * (3 - 2 * fy)
        ix = ix.astype(np.int64)
        iy = iy.astype(np.int64)
        v00 = _hash01(ix, iy, o, seed)
        v10 = _hash01(ix + 1, iy, o, seed)
        v01 = _hash01(ix, iy + 1, o, seed)
        v11 = _hash01(ix + 1, iy + 1, o, seed)
        top = v00 + (v10 - v00) * sx
        bot = v01 + (v11 - v01) * sx
        total += amp * (top + (bot - top) * sy)
        norm += amp
        amp *= persistence
        wl *= 0.5
    return total / norm


@dataclass
class Workload:
    name: str
    model: object
    params: ParameterArrays
    side: float
    config: dict = field(default_factory=dict)


def build_model(n, side, seed, relax):
    b = TerrainModel2DBulider.from_random_sites(n, Site2D(0.0, 0.0), Site2D(side, side), seed=seed)
    if relax:
        b = b.relaxate_sites(relax)
    return b.build()


def border_outlets(model, side, width, sides="all"):
    x, y = model.xs, model.ys
    if sides == "all":
        return (x < width) | (x > side - width) | (y < width) | (y > side - width)
    return (x < width) | (y < width)   # left and bottom


def small(scale=1.0, max_slope=None):
    n = max(16, int(round(10_000 * scale)))
    side = 100.0 * math.sqrt(n / 10_000)
    m = build_model(n, side, 42, 1)
    p = ParameterArrays(n, erodibility=1.0, is_outlet=border_outlets(m, side, 2.0),
                        max_slope=max_slope)
    return Workload("small", m, p, side, {"sites": n, "box": side, "seed": 42, "relax": 1,
                                          "outlets": "border<2.0", "erodibility": "1.0"})


def one_million(scale=1.0):
    n = max(16, int(round(1_000_000 * scale)))
    side = 1000.0 * math.sqrt(n / 1_000_000)
    m = build_model(n, side, 7, 1)
    rng = np.random.default_rng(7)
    v = value_noise(m.xs, m.ys, 7, wavelength=100.0)
    k = np.clip(np.exp(rng.normal(0.0, 0.5, n)) * (0.5 + v), 0.1, 4.0)
    p = ParameterArrays(n, erodibility=k, is_outlet=border_outlets(m, side, 5.0))
    return Workload("1m", m, p, side, {"sites": n, "box": side, "seed": 7, "relax": 1,
                                       "outlets": "border<5.0",
                                       "erodibility": "clamp(exp(N(0,0.5))*(0.5+V4),0.1,4)"})


def sixteen_million(scale=1.0):
    n = max(16, int(round(16_000_000 * scale)))
    side = 4000.0 * math.sqrt(n / 16_000_000)
    m = build_model(n, side, 11, 0)
    v = value_noise(m.xs, m.ys, 11, wavelength=500.0)
    k = 1.0 + 0.8 * (2.0 * v - 1.0)
    p = ParameterArrays(n, erodibility=k, is_outlet=border_outlets(m, side, 5.0, sides="left-bottom"))
    return Workload("16m", m, p, side, {"sites": n, "box": side, "seed": 11, "relax": 0,
                                        "outlets": "left,bottom<5.0",
                                        "erodibility": "1+0.8*(2*V4-1)"})


CONFIGS = {"small": small, "1m": one_million, "16m": sixteen_million}


def _build_many(specs, threads):
    """Models for (n, side, seed) specs, built on a thread pool (the builder's C++
    calls release the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        return list(ex.map(lambda s: build_model(s[0], s[1], s[2], 0), specs))


@dataclass
class BatchWorkload:
    name: str
    models: list
    params: list
    config: dict = field(default_factory=dict)

    @property
    def sites(self):
        return sum(m.num() for m in self.models)


def batched(count=512, lo=4096, hi=262144, seed=3, threads=None):
    """512 independent terrains, site counts log-uniform in [4096, 262144] (seed 3), each
    uniform-random in its own square of side sqrt(n), border outlets within 2% of the
    side, log-normal(0, 0.5) erodibility."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    seeds = rng.integers(1, 2**31, count)
    specs = [(int(n), math.sqrt(n), int(sd)) for n, sd in zip(ns, seeds)]
    models = _build_many(specs, threads or os.cpu_count() or 1)
    params = []
    for (n, side, sd), m in zip(specs, models):
        r = np.random.default_rng(int(sd) + 1)
        k = np.exp(r.normal(0.0, 0.5, n))
        params.append(ParameterArrays(n, erodibility=k, is_outlet=border_outlets(m, side, 0.02 * side)))
    return BatchWorkload("batched", models, params,
                         {"terrains": count, "sites": int(ns.sum()), "n_range": [lo, hi],
                          "seed": seed, "outlets": "border<2% of side",
                          "erodibility": "lognormal(0,0.5)"})



@dataclass
class ServedWorkload:
    name: str
    models: list
    params: list
    arrivals: np.ndarray          # seconds after the first request
    config: dict = field(default_factory=dict)


def served(count=64, rate=200.0, lo=16384, hi=4194304, seed=5, threads=None):
    """A Poisson stream of generate() requests at `rate` per second (seed 5), site counts
    log-uniform in [16384, 4194304], each terrain uniform-random in its own square of
    side sqrt(n) with border outlets within 2% of the side and its own seeded
    erodibility field clamp(exp(N(0,0.5)) * (0.5 + 4-octave value noise), 0.1, 4)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, count)
    arrivals = np.concatenate([[0.0], np.cumsum(gaps[1:])])
    ns = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    seeds = rng.integers(1, 2**31, count)
    specs = [(int(n), math.sqrt(n), int(sd)) for n, sd in zip(ns, seeds)]
    models = _build_many(specs, threads or os.cpu_count() or 1)
    params = []
    for (n, side, sd), m in zip(specs, models):
        r = np.random.default_rng(int(sd) + 1)
        v = value_noise(m.xs, m.ys, int(sd) % 100000, wavelength=max(4.0, side / 8))
        k = np.clip(np.exp(r.normal(0.0, 0.5, n)) * (0.5 + v), 0.1, 4.0)
        params.append(ParameterArrays(n, erodibility=k, is_outlet=border_outlets(m, side, 0.02 * side)))
    return ServedWorkload("served", models, params, arrivals,
                          {"requests": count, "rate_per_s": rate, "sites": int(ns.sum()),
                           "n_range": [lo, hi], "seed": seed})
