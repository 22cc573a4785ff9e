"""Pure-Python restatement of fastlem 0.1.4's solve, for tiny graphs only.

A second, independent restatement next to the C++ oracle (oracle/oracle.cpp): the
tests check that both agree bit for bit, so a slip in either shows up.  Each function
follows the reference lines it names, statement by statement.
"""
import math
import struct

MASK32 = 0xFFFFFFFF
MASK64 = 0xFFFFFFFFFFFFFFFF


# ---- rand 0.8.5 StdRng = ChaCha12 (rand_chacha 0.3), seed_from_u64 (rand_core 0.6) ----

def _rotl(v, c):
    return ((v << c) | (v >> (32 - c))) & MASK32


def chacha_block(key, counter, stream, rounds):
    s = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574, *key,
         counter & MASK32, (counter >> 32) & MASK32, stream & MASK32, (stream >> 32) & MASK32]
    x = list(s)

    def qr(a, b, c, d):
        x[a] = (x[a] + x[b]) & MASK32; x[d] = _rotl(x[d] ^ x[a], 16)
        x[c] = (x[c] + x[d]) & MASK32; x[b] = _rotl(x[b] ^ x[c], 12)
        x[a] = (x[a] + x[b]) & MASK32; x[d] = _rotl(x[d] ^ x[a], 8)
        x[c] = (x[c] + x[d]) & MASK32; x[b] = _rotl(x[b] ^ x[c], 7)

    for _ in range(rounds // 2):
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
    return [(x[i] + s[i]) & MASK32 for i in range(16)]


def seed_from_u64(state):
    MUL, INC = 6364136223846793005, 11634580027462260723
    key = []
    for _ in range(8):
        state = (state * MUL + INC) & MASK64
        xs = (((state >> 18) ^ state) >> 27) & MASK32
        rot = state >> 59
        key.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & MASK32)
    return key


class StdRng:
    def __init__(self, key):
        self.key = key
        self.buf = []
        self.block = 0

    def next_u32(self):
        if not self.buf:
            self.buf = chacha_block(self.key, self.block, 0, 12)
            self.block += 1
        return self.buf.pop(0)

    def next_u64(self):
        lo = self.next_u32()
        hi = self.next_u32()
        return lo | (hi << 32)

    def gen_f64(self):
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))


# ---- std::collections::BinaryHeap<RidgeElement> (stream_tree.rs:15-44, 184) ----

class RustHeap:
    """Max-heap under RidgeElement's reversed Ord: a > b iff a.dist < b.dist."""

    def __init__(self):
        self.data = []

    @staticmethod
    def gt(a, b):
        return b[1] > a[1]

    def le(self, a, b):
        return not self.gt(a, b)

    def push(self, item):
        self.data.append(item)
        self._sift_up(0, len(self.data) - 1)

    def _sift_up(self, start, pos):
        elem = self.data[pos]
        while pos > start:
            parent = (pos - 1) // 2
            if self.le(elem, self.data[parent]):
                break
            self.data[pos] = self.data[parent]
            pos = parent
        self.data[pos] = elem
        return pos

    def pop(self):
        if not self.data:
            return None
        item = self.data.pop()
        if self.data:
            item, self.data[0] = self.data[0], item
            self._sift_down_to_bottom(0)
        return item

    def _sift_down_to_bottom(self, pos):
        end = len(self.data)
        start = pos
        elem = self.data[pos]
        child = 2 * pos + 1
        while child <= max(end - 2, 0) and end >= 2:
            if self.le(self.data[child], self.data[child + 1]):
                child += 1
            self.data[pos] = self.data[child]
            pos = child
            child = 2 * pos + 1
        if child == end - 1:
            self.data[pos] = self.data[child]
            pos = child
        self.data[pos] = elem
        self._sift_up(start, pos)


# ---- the solve (generator.rs, stream_tree.rs, drainage_basin.rs) ----

def neighbors(g, i):
    s, e = int(g.row_ptr[i]), int(g.row_ptr[i + 1])
    return [(int(g.col[k]), float(g.length[k])) for k in range(s, e)]


def has_edge(g, i, j):
    for (jj, w) in neighbors(g, i):
        if jj == j:
            return True, w
    return False, 0.0


def construct_initial_stream_tree(g, elev, is_outlet):          # stream_tree.rs:109-137
    n = g.n
    nxt = list(range(n))
    for i in range(n):
        if is_outlet[i]:
            continue
        steepest = 0.0
        for (j, d) in neighbors(g, i):
            if elev[i] > elev[j]:
                slope = (elev[i] - elev[j]) / d
                if slope > steepest:
                    steepest = slope
                    nxt[i] = j
    return nxt


def find_roots_with_lakes(n, is_outlet, nxt):                    # stream_tree.rs:139-173
    sub = [i if is_outlet[i] else None for i in range(n)]
    has_lake = False
    for i in range(n):
        if sub[i] is not None:
            continue
        iv = i
        while sub[iv] is None and iv != nxt[iv]:
            iv = nxt[iv]
        if sub[iv] is None:
            has_lake = True
            ir = iv
        else:
            ir = sub[iv]
        iv = i
        while sub[iv] is None and iv != nxt[iv]:
            sub[iv] = ir
            iv = nxt[iv]
        sub[iv] = ir
    return sub, has_lake


def remove_lakes(g, nxt, outlets, sub):                          # stream_tree.rs:175-243
    n = g.n
    root = [None] * n
    heap = RustHeap()
    for o in outlets:
        root[o] = o
        heap.push((o, 0.0))
    visited = [False] * n
    nxt = list(nxt)
    while True:
        el = heap.pop()
        if el is None:
            break
        i = el[0]
        if visited[i]:
            continue
        for (j, d) in neighbors(g, i):
            if visited[j]:
                continue
            if root[sub[j]] is None:
                k, nk = j, i
                while nxt[k] != k:
                    tmp = nxt[k]
                    nxt[k] = nk
                    nk = k
                    k = tmp
                nxt[k] = nk
                root[sub[j]] = root[sub[i]]
            heap.push((j, d))
        root[i] = root[sub[i]]
        visited[i] = True
    return nxt


def stream_tree(g, elev, outlets):                               # stream_tree.rs:72-99
    is_out = [False] * g.n
    for o in outlets:
        is_out[o] = True
    nxt = construct_initial_stream_tree(g, elev, is_out)
    sub, has_lake = find_roots_with_lakes(g.n, is_out, nxt)
    if not has_lake:
        return nxt, False
    return remove_lakes(g, nxt, outlets, sub), True


def drainage_basin(g, nxt, outlet):                              # drainage_basin.rs:13-36
    trav = [outlet]
    i = 0
    while True:
        it = trav[i]
        for (jt, _) in neighbors(g, it):
            if nxt[jt] == it:
                trav.append(jt)
        i += 1
        if i >= len(trav):
            break
    return trav


def generate(g, base, k, u, is_outlet, max_slope=None, max_iteration=None):  # generator.rs:90-213
    n = g.n
    outlets = [i for i in range(n) if is_outlet[i]]
    if not outlets:
        outlets = [int(o) for o in g.default_outlets]
    rng = StdRng(seed_from_u64(0))
    eps = 2.220446049250313e-16
    elev = [float(base[i]) + rng.gen_f64() * eps for i in range(n)]
    iters = 0
    limit = 0xFFFFFFFF if max_iteration is None else max_iteration
    trace = []
    for _ in range(limit):
        iters += 1
        nxt, _ = stream_tree(g, elev, outlets)
        drain = [float(a) for a in g.area]
        resp = [0.0] * n
        changed = False
        for outlet in outlets:
            trav = drainage_basin(g, nxt, outlet)
            for i in reversed(trav):
                j = nxt[i]
                if j != i:
                    drain[j] += drain[i]
            for i in trav:
                j = nxt[i]
                ok, e = has_edge(g, i, j)
                distance = e if ok else 1.0
                celerity = float(k[i]) * math.sqrt(drain[i])
                resp[i] += resp[j] + 1.0 / celerity * distance
            for i in trav:
                dt = resp[i] - resp[outlet]
                new_e = elev[outlet] + float(u[i]) * (dt if dt > 0.0 else 0.0)
                if max_slope is not None and not math.isnan(max_slope[i]):
                    j = nxt[i]
                    ok, e = has_edge(g, i, j)
                    distance = e if ok else 1.0
                    ms = math.tan(max_slope[i])
                    slope = (new_e - elev[j]) / distance
                    if slope > ms:
                        new_e = elev[j] + ms * distance
                changed |= new_e != elev[i]
                elev[i] = new_e
        trace.append(list(nxt))
        if not changed:
            break
    return elev, iters, trace


def f64_bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]
