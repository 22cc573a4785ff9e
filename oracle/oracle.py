"""ctypes front end of the CPU oracle (test infrastructure, not the product).

Every function mirrors one step of fastlem 0.1.4's solve; the C++ source
(oracle/oracle.cpp) cites the reference lines each one restates.
"""
import ctypes
import numpy as np

from . import build as _build

_lib = None

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.build())
        c_u32, c_u64, c_int = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        vp = ctypes.c_void_p
        L.orc_rng_f64.argtypes = [c_u64, c_u64, c_u64, f64p]
        L.orc_chacha_block.argtypes = [u32p, c_u64, c_u64, c_int, u32p]
        L.orc_seed_from_u64.argtypes = [c_u64, u32p]
        L.orc_resolve_outlets.argtypes = [c_u32, u8p, u32p, c_u32, u32p]
        L.orc_resolve_outlets.restype = c_u32
        L.orc_initial_tree.argtypes = [c_u32, u32p, u32p, f64p, f64p, u8p, u32p]
        L.orc_roots.argtypes = [c_u32, u8p, u32p, u32p]
        L.orc_roots.restype = c_int
        L.orc_remove_lakes_heap.argtypes = [c_u32, u32p, u32p, f64p, u32p, c_u32, u32p, u32p]
        L.orc_remove_lakes_heap.restype = c_int
        L.orc_prim_rank.argtypes = [c_u32, u32p, u32p, f64p, u32p, c_u32, u32p]
        L.orc_prim_rank.restype = c_int
        L.orc_remove_lakes_rank.argtypes = [c_u32, u32p, u32p, u8p, u32p, u32p, u32p]
        L.orc_tree_pass.argtypes = [c_u32, u32p, u32p, f64p, f64p, u32p, c_u32,
                                    f64p, f64p, f64p, c_int, u32p, f64p, f64p, f64p]
        L.orc_tree_pass.restype = c_int
        L.orc_generate.argtypes = [c_u32, u32p, u32p, f64p, f64p, u32p, c_u32,
                                   f64p, f64p, f64p, u8p, vp, c_u32, c_int, f64p,
                                   ctypes.POINTER(c_u32), c_u32, vp, vp, vp,
                                   ctypes.POINTER(ctypes.c_double)]
        L.orc_generate.restype = c_int
        L.orc_pow_sqrt_mismatches.argtypes = [f64p, c_u64]
        L.orc_pow_sqrt_mismatches.restype = c_u64
        _lib = L
    return _lib


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def rng_f64(count, seed=0, first=0):
    """`StdRng::seed_from_u64(seed)` then `count` draws of `gen::<f64>()`."""
    out = np.empty(count, np.float64)
    lib().orc_rng_f64(seed, first, count, out)
    return out


def chacha_block(key_words, counter, stream, rounds):
    out = np.empty(16, np.uint32)
    lib().orc_chacha_block(_u32(key_words), counter, stream, rounds, out)
    return out


def seed_from_u64(seed):
    out = np.empty(8, np.uint32)
    lib().orc_seed_from_u64(seed, out)
    return out


def resolve_outlets(is_outlet, default_outlets):
    is_outlet = _u8(is_outlet)
    d = _u32(default_outlets)
    out = np.empty(max(len(is_outlet), len(d), 1), np.uint32)
    c = lib().orc_resolve_outlets(len(is_outlet), is_outlet, d, len(d), out)
    return out[:c].copy()


def initial_tree(g, elev, outlet_table):
    nxt = np.empty(g.n, np.uint32)
    lib().orc_initial_tree(g.n, g.row_ptr, g.col, g.length, _f64(elev), _u8(outlet_table), nxt)
    return nxt


def roots(outlet_table, nxt):
    nxt = _u32(nxt)
    sub = np.empty(len(nxt), np.uint32)
    has_lake = lib().orc_roots(len(nxt), _u8(outlet_table), nxt, sub)
    return sub, bool(has_lake)


def remove_lakes_heap(g, nxt, outlets, subroot):
    out = _u32(nxt).copy()
    o = _u32(outlets)
    rc = lib().orc_remove_lakes_heap(g.n, g.row_ptr, g.col, g.length, o, len(o), _u32(subroot), out)
    if rc != 0:
        raise ValueError("NaN edge length")
    return out


def prim_rank(g, outlets):
    o = _u32(outlets)
    rank = np.empty(g.n, np.uint32)
    rc = lib().orc_prim_rank(g.n, g.row_ptr, g.col, g.length, o, len(o), rank)
    if rc != 0:
        raise ValueError("NaN edge length")
    return rank


def remove_lakes_rank(g, nxt, outlet_table, subroot, rank):
    out = _u32(nxt).copy()
    lib().orc_remove_lakes_rank(g.n, g.row_ptr, g.col, _u8(outlet_table), _u32(subroot),
                                _u32(rank), out)
    return out


def tree_pass(g, nxt, outlets, k, u, tanms, elev, use_pow=False):
    """Returns (changed, elev_new, drainage, response) for one pass on receivers `nxt`."""
    e = _f64(elev).copy()
    drain = np.empty(g.n, np.float64)
    resp = np.empty(g.n, np.float64)
    o = _u32(outlets)
    ch = lib().orc_tree_pass(g.n, g.row_ptr, g.col, g.length, g.area, o, len(o), _f64(k), _f64(u),
                             _f64(tanms), int(use_pow), _u32(nxt), e, drain, resp)
    return bool(ch), e, drain, resp


def generate(g, base, k, u, is_outlet, max_slope=None, max_iter=0, use_pow=False,
             use_rank=False, trace_cap=0):
    """fastlem generate() on graph `g`.  Returns a dict with elev, iters, seconds and,
    when trace_cap > 0, per-iteration receivers / elevations / has_lake."""
    n = g.n
    out = np.empty(n, np.float64)
    iters = ctypes.c_uint32(0)
    secs = ctypes.c_double(0.0)
    ms = None if max_slope is None else _f64(max_slope)
    tn = te = tl = None
    if trace_cap:
        tn = np.zeros((trace_cap, n), np.uint32)
        te = np.zeros((trace_cap, n), np.float64)
        tl = np.zeros(trace_cap, np.uint8)
    flags = (1 if use_pow else 0) | (2 if use_rank else 0)
    vp = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
    rc = lib().orc_generate(n, g.row_ptr, g.col, g.length, g.area, g.default_outlets,
                            len(g.default_outlets), _f64(base), _f64(k), _f64(u), _u8(is_outlet),
                            vp(ms), max_iter, flags, out, ctypes.byref(iters), trace_cap,
                            vp(tn), vp(te), vp(tl), ctypes.byref(secs))
    if rc != 0:
        raise ValueError("NaN edge length")
    res = {"elev": out, "iters": iters.value, "seconds": secs.value}
    if trace_cap:
        m = min(iters.value, trace_cap)
        res["trace_next"] = tn[:m]
        res["trace_elev"] = te[:m]
        res["trace_has_lake"] = tl[:m].astype(bool)
    return res


def pow_sqrt_mismatches(vals):
    v = _f64(vals)
    return int(lib().orc_pow_sqrt_mismatches(v, len(v)))
