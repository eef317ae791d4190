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
