"""The exact parallel fold used by the chain walks (csrc/fold.cuh) against a plain
sequential accumulation: every partial sum must be bit-identical."""
import numpy as np
import pytest

from fastlem_gb300._lib import check, lib, ptr

pytestmark = pytest.mark.gpu


def sequential(start, ops):
    out = np.empty(len(ops))
    x = start
    for i, y in enumerate(ops):
        x = x + y                      # one IEEE rounding per addition, in order
        out[i] = x
    return out


def gpu_fold(start, ops):
    ops = np.ascontiguousarray(ops, np.float64)
    out = np.empty(len(ops))
    check(lib().fl_probe_chain_fold(ptr(ops), len(ops), float(start), ptr(out)))
    return out


def cases():
    rng = np.random.default_rng(12)
    yield "log-uniform", 1.0, np.exp(rng.uniform(-20, 3, 5000))
    yield "small-into-large", 1e6, rng.uniform(0, 1, 5000)
    yield "crossings", 1e-3, np.full(4000, 1e-3) * rng.uniform(0.5, 1.5, 4000)
    # exact half-ulp operands: ties to even at every step
    yield "ties", 1.0, np.full(3000, 2.0 ** -53)
    yield "mixed-ties", 1.0, rng.integers(0, 8, 3000) * 2.0 ** -54
    yield "zeros-subnormals", 1e-300, np.concatenate([np.zeros(50), np.full(50, 5e-324),
                                                     np.full(50, 1e-310), rng.uniform(0, 1e-300, 50)])
    yield "from-zero", 0.0, rng.uniform(0, 1, 200)
    yield "negative-operands", 10.0, rng.uniform(-1, 1, 2000)
    yield "non-finite", 1.0, np.array([1.0, np.inf, 2.0, -np.inf, np.nan, 1.0])
    yield "long-river", 0.37, rng.uniform(0.01, 0.02, 40000)
    # cell areas that lost their low bits to cancellation (granularity 2^-30) added to
    # a drainage area crossing 2^23 and 2^24: ties with a parity-dependent outcome
    yield "coarse-areas", 2.0 ** 23 - 3000.0, 1.0 + rng.integers(0, 2 ** 20, 30000) * 2.0 ** -30
    yield "short", 2.5, np.array([0.25])


@pytest.mark.parametrize("name,start,ops", list(cases()), ids=[c[0] for c in cases()])
def test_fold_matches_sequential_accumulation(name, start, ops):
    with np.errstate(invalid="ignore"):
        want = sequential(start, ops)
    got = gpu_fold(start, ops)
    g, w = got.view(np.uint64), want.view(np.uint64)
    # bit-identical, except that the payload of a NaN is the platform's own choice
    bad = np.nonzero((g != w) & ~(np.isnan(got) & np.isnan(want)))[0]
    assert len(bad) == 0, f"{name}: {len(bad)} partial sums differ, first at {bad[:3]}"
