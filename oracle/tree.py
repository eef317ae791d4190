"""numpy restatement of the reference's tree DP executor (test infrastructure only).

join(...)    one join over all 2^J compatible pairs, cdist/tree_dp.c:13-39 (the Gray-code order of
             the reference visits every pair once, so the minimum is order independent)
run(prog, t) the post-order stack executor of cdist/tree_dp.py:442-501 over a compiled tree (the
             product's CompiledTreeDP supplies the interfaces and generator maps; the compilation
             is pinned separately by the reference's own results in tests/golden/tree_dp.json)
brute_affine / brute_logical   exhaustive minima (tests/test_tree_dp.py:45-69)
"""
from __future__ import annotations

from itertools import product

import numpy as np


def join(left, right, lmaps, rmaps, parent_rank, inf):
    """Parent table: min over pairs x of left[L(x)] + right[R(x)], parent index x & (2^P - 1)."""
    J = len(lmaps)
    li = np.zeros(1, dtype=np.int64)
    ri = np.zeros(1, dtype=np.int64)
    for b in range(J):                     # states of all x by doubling: bit b toggles map b
        li = np.concatenate([li, li ^ np.int64(lmaps[b])])
        ri = np.concatenate([ri, ri ^ np.int64(rmaps[b])])
    a = left[li].astype(np.int64)
    c = right[ri].astype(np.int64)
    ok = (a < inf) & (c < inf) & (a <= inf - c)
    out = np.full(1 << parent_rank, inf, dtype=np.int64)
    x = np.arange(1 << J, dtype=np.int64)
    np.minimum.at(out, (x & ((1 << parent_rank) - 1))[ok], (a + c)[ok])
    return out


def run(prog, target):
    """Exact minimum weight for M e = target through the compiled tree, or None."""
    rep = prog.representative(target)
    if rep is None:
        return None
    if not prog.nodes:
        return 0
    inf = prog.infinity
    tabs = {}
    for i in prog.order:
        nd = prog.nodes[i]
        size = 1 << len(prog.interfaces[i])
        if nd.leaf is not None:
            t = np.full(size, inf, dtype=np.int64)
            bit = (rep >> nd.leaf) & 1
            t[0] = bit if prog.columns[nd.leaf] else 0
            if size == 2:
                t[1] = bit ^ 1
            tabs[i] = t
            continue
        jn = prog.joins[i]
        lo = (1 << jn.left_rank) - 1
        gens = jn.parent_maps + jn.free_maps
        tabs[i] = join(tabs.pop(nd.left), tabs.pop(nd.right), [g & lo for g in gens],
                       [g >> jn.left_rank for g in gens], jn.parent_rank, inf)
    v = int(tabs[prog.root][0])
    assert v < inf, "a consistent affine system must have a finite root cost"
    return v


def node_tables(prog, target):
    """Every node's table (index -> int64 array) for the target (for table-by-table checks)."""
    rep = prog.representative(target)
    inf = prog.infinity
    tabs = {}
    for i, nd in enumerate(prog.nodes):
        size = 1 << len(prog.interfaces[i])
        if nd.leaf is not None:
            t = np.full(size, inf, dtype=np.int64)
            bit = (rep >> nd.leaf) & 1
            t[0] = bit if prog.columns[nd.leaf] else 0
            if size == 2:
                t[1] = bit ^ 1
            tabs[i] = t
            continue
        jn = prog.joins[i]
        lo = (1 << jn.left_rank) - 1
        gens = jn.parent_maps + jn.free_maps
        tabs[i] = join(tabs[nd.left], tabs[nd.right], [g & lo for g in gens], [g >> jn.left_rank for g in gens],
                       jn.parent_rank, inf)
    return tabs


def brute_affine(columns):
    """Least weight of every reachable target over all 2^n assignments."""
    out = {}
    for bits in product((0, 1), repeat=len(columns)):
        t = 0
        for b, c in zip(bits, columns):
            if b:
                t ^= c
        out[t] = min(out.get(t, len(columns) + 1), sum(bits))
    return out


def brute_logical(h, l, mask):
    best = None
    for bits in product((0, 1), repeat=len(h)):
        s = g = 0
        for b, hc, lc in zip(bits, h, l):
            if b:
                s ^= hc
                g ^= lc
        if s == 0 and bin(g & mask).count("1") % 2:
            w = sum(bits)
            best = w if best is None else min(best, w)
    return best


_PORT = None


def port_lib():
    """oracle/tree_port.so (built by oracle/Makefile)."""
    global _PORT
    if _PORT is None:
        import ctypes
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tree_port.so")
        L = ctypes.CDLL(path)
        for b in (8, 16, 32):
            f = getattr(L, "tree_join_port_u%d" % b)
            f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_uint] + [ctypes.c_uint64] * 3
            f.restype = None
        _PORT = L
    return _PORT


def run_port(prog, target, chunk=1 << 20):
    """The reference's executor (cdist/tree_dp.py:442-501: one arena of the table dtype in post-order
    with stack compaction, joins in chunks of 2^20 pairs) over the C port of its join: the timed
    single-threaded CPU baseline.  Returns the minimum weight or None."""
    rep = prog.representative(target)
    if rep is None:
        return None
    if not prog.nodes:
        return 0
    L = port_lib()
    dt = np.dtype(prog.dtype)
    fn = getattr(L, "tree_join_port_u%d" % (8 * dt.itemsize))
    inf = prog.infinity
    arena = np.empty(prog.peak_live_entries, dtype=dt)
    base, item = arena.ctypes.data, dt.itemsize
    gl = np.empty(64, dtype=np.uint64)
    gr = np.empty(64, dtype=np.uint64)
    stack, live = [], 0
    for i in prog.order:
        nd = prog.nodes[i]
        size = 1 << len(prog.interfaces[i])
        out = arena[live:live + size]
        out.fill(inf)
        if nd.leaf is not None:
            bit = (rep >> nd.leaf) & 1
            out[0] = bit if prog.columns[nd.leaf] else 0
            if size == 2:
                out[1] = bit ^ 1
            stack.append((i, live, size))
            live += size
            continue
        b, a = stack.pop(), stack.pop()
        left, right = (a, b) if a[0] == nd.left else (b, a)
        jn = prog.joins[i]
        lo = (1 << jn.left_rank) - 1
        gens = jn.parent_maps + jn.free_maps
        for k, g in enumerate(gens):
            gl[k] = g & lo
            gr[k] = g >> jn.left_rank
        for s in range(0, jn.work, chunk):
            fn(base + left[1] * item, base + right[1] * item, base + live * item, gl.ctypes.data, gr.ctypes.data,
               jn.parent_rank, s, min(s + chunk, jn.work), inf)
        dst = a[1]
        arena[dst:dst + size] = arena[live:live + size].copy()
        live = dst + size
        stack.append((i, dst, size))
    v = int(arena[0])
    assert v < inf
    return v
