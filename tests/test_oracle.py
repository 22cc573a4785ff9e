"""CPU tests of the oracle: published ChaCha vectors, agreement with the pure-Python
restatement, the rank-based lake re-routing against the heap-driven one, and the
committed golden vectors."""
import json
import math
import os

import numpy as np
import pytest

from tests import graphs, pyref

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_chacha20_rfc7539_block(orc):
    # RFC 7539 section 2.3.2: key 00..1f, nonce 00:00:00:09:00:00:00:4a:00:00:00:00,
    # block counter 1, 20 rounds.  The IETF layout (32-bit counter, 96-bit nonce) maps
    # onto the 64-bit counter / 64-bit stream layout as counter = 1 | 0x09000000 << 32,
    # stream = 0x4a000000.
    key = np.array([int.from_bytes(bytes(range(4 * i, 4 * i + 4)), "little") for i in range(8)],
                   np.uint32)
    out = orc.chacha_block(key, 1 | (0x09000000 << 32), 0x4A000000, 20)
    assert [hex(v) for v in out[:4]] == ["0xe4e7f110", "0x15593bd1", "0x1fdd0f50", "0xc47120a3"]
    assert list(out) == pyref.chacha_block([int(v) for v in key], 1 | (0x09000000 << 32), 0x4A000000, 20)


def test_chacha20_zero_key_keystream(orc):
    # The all-zero key / nonce / counter ChaCha20 keystream starts 76 b8 e0 ad a0 f1 3d 90.
    out = orc.chacha_block(np.zeros(8, np.uint32), 0, 0, 20)
    assert bytes(np.asarray(out[:2], "<u4").tobytes()) == bytes.fromhex("76b8e0ada0f13d90")


def test_rng_matches_python_restatement(orc):
    key = pyref.seed_from_u64(0)
    assert list(orc.seed_from_u64(0)) == key
    rng = pyref.StdRng(key)
    ref = [rng.gen_f64() for _ in range(40)]
    got = orc.rng_f64(40)
    assert [pyref.f64_bits(x) for x in ref] == [pyref.f64_bits(x) for x in got]
    # random access into the keystream
    assert np.array_equal(orc.rng_f64(13, first=27), got[27:40])
    assert all(0.0 <= x < 1.0 for x in got)


def test_heap_pop_order_matches_python(orc):
    # prim_rank drives the C++ heap; the pure-Python heap replays the same pushes.
    for seed in range(5):
        g = graphs.grid(6, 5, unit_lengths=(seed % 2 == 0), jitter=0.2, seed=seed)
        outlets = list(g.default_outlets)
        rank = orc.prim_rank(g, np.array(outlets, np.uint32))
        heap = pyref.RustHeap()
        for o in outlets:
            heap.push((o, 0.0))
        visited = [False] * g.n
        order = []
        while True:
            el = heap.pop()
            if el is None:
                break
            i = el[0]
            if visited[i]:
                continue
            for (j, d) in pyref.neighbors(g, i):
                if not visited[j]:
                    heap.push((j, d))
            visited[i] = True
            order.append(i)
        expect = np.full(g.n, 0xFFFFFFFF, np.uint32)
        expect[np.array(order)] = np.arange(len(order))
        assert np.array_equal(rank, expect)


def _cases():
    yield "line", graphs.line(7), None
    yield "star", graphs.star(5), None
    yield "grid_ties", graphs.grid(5, 4, unit_lengths=True, seed=1), None
    yield "grid_jitter", graphs.grid(6, 6, jitter=0.3, seed=2), None
    yield "two_components", graphs.two_components(), None
    yield "grid_slope", graphs.grid(6, 5, jitter=0.3, seed=3), 0.314


@pytest.mark.parametrize("name,g,ms", list(_cases()), ids=[c[0] for c in _cases()])
def test_oracle_matches_python_restatement(orc, name, g, ms):
    n = g.n
    rng = np.random.default_rng(7)
    base = np.zeros(n) if name != "grid_jitter" else rng.uniform(0, 0.1, n)
    k = rng.uniform(0.5, 2.0, n)
    u = np.ones(n) if name != "grid_jitter" else rng.uniform(0.5, 1.5, n)
    is_out = np.zeros(n, np.uint8)
    max_slope = None if ms is None else np.full(n, ms)
    ref_e, ref_it, ref_trace = pyref.generate(g, base, k, u, is_out, max_slope)
    for use_rank in (False, True):
        r = orc.generate(g, base, k, u, is_out, max_slope=max_slope, use_rank=use_rank, trace_cap=64)
        assert r["iters"] == ref_it
        assert [pyref.f64_bits(x) for x in r["elev"]] == [pyref.f64_bits(x) for x in ref_e]
        for it, nxt in enumerate(ref_trace[:64]):
            assert list(r["trace_next"][it]) == nxt


def test_rank_reformulation_equals_heap_on_random_graphs(orc):
    """The per-lake (rank, slot) minimum reproduces the heap's re-routing exactly."""
    for seed in range(12):
        if seed % 3 == 0:
            g = graphs.grid(9, 7, unit_lengths=True, seed=seed)        # many equal keys
        else:
            g = graphs.random_delaunay(300, seed)
        rng = np.random.default_rng(seed)
        elev = rng.uniform(0, 1, g.n)
        if seed % 2:
            elev = np.round(elev * 4) / 4                               # equal elevations
        outlets = np.array(sorted(rng.choice(g.n, size=max(1, g.n // 40), replace=False)), np.uint32)
        if seed % 4 == 1:
            outlets = outlets[::-1].copy()                              # order matters for ties
        table = np.zeros(g.n, np.uint8)
        table[outlets] = 1
        nxt = orc.initial_tree(g, elev, table)
        sub, has_lake = orc.roots(table, nxt)
        assert has_lake
        by_heap = orc.remove_lakes_heap(g, nxt, outlets, sub)
        rank = orc.prim_rank(g, outlets)
        by_rank = orc.remove_lakes_rank(g, nxt, table, sub, rank)
        assert np.array_equal(by_heap, by_rank)


def test_max_iteration_bounds(orc):
    g = graphs.grid(5, 5, jitter=0.2, seed=4)
    n = g.n
    args = (np.zeros(n), np.ones(n), np.ones(n), np.zeros(n, np.uint8))
    r0 = orc.generate(g, *args, max_iter=0)
    # set_max_iteration(0) is handled by the caller; the oracle treats 0 as unset
    full = orc.generate(g, *args)
    r1 = orc.generate(g, *args, max_iter=1)
    assert r1["iters"] == 1
    assert full["iters"] >= 1 and r0["iters"] == full["iters"]


def test_golden_vectors(orc):
    """The committed oracle outputs (tests/golden/make_golden.py) still reproduce."""
    with open(os.path.join(GOLDEN, "small_graphs.json")) as f:
        cases = json.load(f)
    assert cases
    for c in cases:
        g = graphs.from_csr(c)
        ms = None if c["max_slope"] is None else np.array(c["max_slope"], np.float64)
        r = orc.generate(g, np.array(c["base"]), np.array(c["k"]), np.array(c["u"]),
                         np.array(c["is_outlet"], np.uint8), max_slope=ms)
        assert r["iters"] == c["iters"], c["name"]
        assert [pyref.f64_bits(x) for x in r["elev"]] == [int(b, 16) for b in c["elev_bits"]], c["name"]
