"""Completion tables of the weight-bounded search, built and probed on the GPU (drop-in for the
table part of cdist/search.py; the depth-first search itself stays with the caller).

row_hashes / column_hashes   128-bit XOR-linear syndrome hashes, seeded as cdist/search.py:83-105
Table(p, k)                  all column subsets of size <= k keyed by syndrome hash, on the device
                             (cdist/search.py:108-142; cdist/gmitm.c:61-186)
Table.lookup(...)            batched probes: least cost <= R with the same fingerprint and another
                             logical label (cdist/gmitm.c:138-163)
"""
from __future__ import annotations

import ctypes
import math
import random
import time

import numpy as np

from . import _lib, device
from .problem import Problem

DMAX = 40               # deepest threshold of the reference's search kernel (cdist/search.py:18)


def check_threshold(K):
    if K > DMAX:
        raise ValueError(f"threshold {K} exceeds the search depth {DMAX} of the kernel; nothing can be "
                         "concluded at this threshold")


def row_hashes(nrows, seed):
    """Two 64-bit random words per row from random.Random(seed) (cdist/search.py:83-85)."""
    rng = random.Random(seed)
    return ([rng.getrandbits(64) for _ in range(nrows)], [rng.getrandbits(64) for _ in range(nrows)])


def column_hashes(h, rh):
    """XOR of the row words over each column's rows: (zh, zl) uint64 arrays."""
    zh = np.zeros(len(h), dtype=np.uint64)
    zl = np.zeros(len(h), dtype=np.uint64)
    cache = {}
    for j, a in enumerate(h):
        v = cache.get(a)
        if v is None:
            x = y = 0
            m = a
            while m:
                low = m & -m
                r = low.bit_length() - 1
                x ^= rh[0][r]
                y ^= rh[1][r]
                m ^= low
            v = cache[a] = (x, y)
        zh[j], zl[j] = v
    return zh, zl


class Table:
    """All column subsets of size <= k of a problem, keyed by syndrome hash, in device memory."""

    def __init__(self, p: Problem, k, seed=12345, load=0.5, labelfree=False):
        assert labelfree or p.nobs <= 64, "more than 64 observables need a label-free table"
        device.require_gpu()
        self.problem = p
        self.k = k
        self.labelfree = labelfree
        self.wide = p.nobs > 16 and not labelfree
        self.rh = row_hashes(p.nrows, seed)
        self.zh, self.zl = column_hashes(p.h, self.rh)
        self.lg = np.zeros(p.ncols, dtype=np.uint64) if labelfree else np.array(p.l, dtype=np.uint64)
        n = p.ncols
        total = sum(math.comb(n, i) for i in range(k + 1))
        self.log2slots = max(10, math.ceil(math.log2(total / load + 1)))
        L = _lib.lib()
        st = ctypes.c_int(0)
        self.handle = L.tg_tab_create(self.log2slots, 1 if self.wide else 0, ctypes.byref(st))
        if not self.handle:
            if st.value == -3:
                raise MemoryError(f"table with 2^{self.log2slots} slots")
            _lib.check(st.value)
        t = time.time()
        _lib.check(L.tg_tab_build(self.handle, n, self.zh.ctypes.data, self.zl.ctypes.data, self.lg.ctypes.data, k))
        self.build_seconds = time.time() - t
        self.entries = int(L.tg_tab_count(self.handle))

    def hashes_for(self, h):
        """Hashes of arbitrary syndromes of this table's problem."""
        return column_hashes(h, self.rh)

    def lookup(self, zh, zl, lg, R):
        """Batched probes: per probe the least cost <= R[q] of a subset with the probe's syndrome
        hash and a logical label other than lg[q], or -1.  A label-free table stores label 0 and is
        probed with label 1, so every entry qualifies (as cdist/gmitm.c:618, 1046 do)."""
        import torch
        zh, zl = np.asarray(zh, dtype=np.uint64), np.asarray(zl, dtype=np.uint64)
        lg = np.ones(zh.size, dtype=np.uint64) if self.labelfree else np.asarray(lg, dtype=np.uint64)
        R = np.broadcast_to(np.asarray(R, dtype=np.int32), zh.shape)
        m = zh.size
        if m == 0:
            return np.zeros(0, dtype=np.int32)
        dev = [torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda() for a in (zh, zl, lg)]
        r = torch.from_numpy(np.array(R, dtype=np.int32)).cuda()
        out = torch.empty(m, dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().tg_tab_lookup_dev(self.handle, m, dev[0].data_ptr(), dev[1].data_ptr(),
                                                dev[2].data_ptr(), r.data_ptr(), out.data_ptr(), device.stream_ptr()))
        return out.cpu().numpy()

    def lookup_syndromes(self, syndromes, labels, R):
        """lookup() for syndromes given as row bitmasks."""
        zh, zl = self.hashes_for(list(syndromes))
        return self.lookup(zh, zl, labels, R)

    def free(self):
        if self.handle:
            _lib.lib().tg_tab_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------------- the search
def _search_arrays(p: Problem):
    """Columns as W-word syndromes, rows -> columns and columns -> rows (CSR), largest column weight."""
    from .trellis import bit_positions
    n, m = p.ncols, p.nrows
    W = max(1, (m + 63) // 64)
    col = np.frombuffer(b"".join(int(a).to_bytes(8 * W, "little") for a in p.h), dtype=np.uint64).reshape(n, W) \
        if n else np.zeros((0, W), dtype=np.uint64)
    col_start, col_rows = bit_positions(list(p.h), m)
    entry_col = np.repeat(np.arange(n, dtype=np.int32), np.diff(col_start))
    o = np.argsort(col_rows, kind="stable")
    row_cols = entry_col[o].astype(np.int32)
    row_start = np.zeros(m + 1, dtype=np.int64)
    row_start[1:] = np.cumsum(np.bincount(col_rows, minlength=m))[:m]
    wmax = int(np.diff(col_start).max()) if n else 1
    return (W, np.ascontiguousarray(col), row_start.astype(np.int32), np.ascontiguousarray(row_cols),
            col_start.astype(np.int32), np.ascontiguousarray(col_rows.astype(np.int32)), max(1, wmax))


def partners(p: Problem, row_start=None, row_cols=None):
    """Each column's partners: the columns y sharing a row with f such that f ^ y is again a column
    with the XOR of their labels (cdist/search.py:207-231; a minimum logical never holds both f and
    y).  Returns (ex_start int32 [n + 1], ex_cols int32), and the number of pairs."""
    if row_start is None:
        _, _, row_start, row_cols, _, _, _ = _search_arrays(p)
    index = {(int(a), int(b)): j for j, (a, b) in enumerate(zip(p.h, p.l))}
    part = [set() for _ in range(p.ncols)]
    seen = set()
    for r in range(p.nrows):
        cols = row_cols[row_start[r]:row_start[r + 1]].tolist()
        for i, x in enumerate(cols):
            for y in cols[i + 1:]:
                if (x, y) in seen:
                    continue
                seen.add((x, y))
                z = index.get((int(p.h[x]) ^ int(p.h[y]), int(p.l[x]) ^ int(p.l[y])))
                if z is not None:
                    part[x].update((y, z))
                    part[y].update((x, z))
                    part[z].update((x, y))
    ex_start = np.zeros(p.ncols + 1, dtype=np.int32)
    ex_start[1:] = np.cumsum([len(x) for x in part])
    ex_cols = np.array([y for x in part for y in sorted(x)] or [0], dtype=np.int32)
    return ex_start, ex_cols, int(ex_start[-1]) // 2


def distance(p: Problem, k_table=2, kmax=20, relaxed=None, rank=None, anchors=None, enum_all=False, time_limit=0.0,
             log=None, start=1, exclusions=True, on_run=None, table_load=0.5, kernel=None, cover=False,
             labelfree=None, wave=1 << 16, probe=None, seed=12345, threads=1, probe_fn=None, probe_ctx=None):
    """Exact distance by iterative deepening over the threshold K (cdist/search.py:387-441): per K a
    depth-first search over column sets, the completion table of all subsets of at most k_table
    columns answering the last levels (tg_search; the probes of many nodes go to the device table in
    one wave of up to `wave` probes).  Returns the reference's record: k_table, table_entries,
    table_seconds, runs (per K: status, best, nodes, lookups, hits, false_hits, seconds),
    lower_bound, distance (None if none <= kmax), solutions, solutions_complete.

    exclusions: forbid each taken column's partners below it (as the reference); cover: the covering
    bound (True / "ascent", or "simple" without the ascent; off by default, as the reference's);
    kernel (the reference's kernel dominance) is accepted and not applied (the result does not
    depend on it).  enum_all, relaxed tables and label-free search (more than 64
    observables) are not provided.  probe: a callable (zh, zl, lg, R) -> costs answering the probes
    instead of the device table (the tests plug in the oracle's table).  threads: host threads that
    share out the anchors of each threshold (the probes still go out one wave at a time).
    probe_fn / probe_ctx: a native tg_probe_fn (a _sigs_extra.PROBE_FN) and its context answering the
    probes instead (a host table: the timed CPU baseline)."""
    import ctypes
    from ._sigs_extra import PROBE_FN
    if enum_all or relaxed:
        raise NotImplementedError("enum_all and relaxed tables are not provided by this search")
    if labelfree or p.nobs > 64:
        raise NotImplementedError("label-free search (more than 64 observables) is not provided")
    W, col, row_start, row_cols, col_start, col_rows, wmax = _search_arrays(p)
    n = p.ncols
    # cover: False, True / "ascent" (the covering bound with its dual ascent), "simple" (first dual)
    cover_mode = 0 if not cover else (1 if cover == "simple" else 2)
    ex_start = ex_cols = None
    n_excl = 0
    if exclusions and n:
        ex_start, ex_cols, n_excl = partners(p, row_start, row_cols)
    rank_a = np.ascontiguousarray(np.asarray(rank if rank is not None else range(n), dtype=np.int32))
    anch = np.ascontiguousarray(np.asarray(anchors if anchors is not None else range(n), dtype=np.int32))
    lg = np.ascontiguousarray(np.array([int(x) for x in p.l], dtype=np.uint64)) if n else np.zeros(1, np.uint64)
    table = None
    out = {"k_table": k_table, "table_entries": None, "table_seconds": 0.0, "exclusion_pairs": n_excl, "runs": [],
           "lower_bound": start, "distance": None, "solutions": [], "solutions_complete": False}
    if probe_fn is not None:
        zh, zl = column_hashes(p.h, row_hashes(p.nrows, seed))
        look = None
    elif probe is None:
        table = Table(p, k_table, seed=seed, load=table_load)
        zh, zl = table.zh, table.zl
        look = table.lookup
        out["table_entries"], out["table_seconds"] = table.entries, table.build_seconds
        if log:
            log(f"  table k={k_table}: {table.entries} entries in 2^{table.log2slots} slots "
                f"({table.build_seconds:.1f}s)")
    else:
        zh, zl = column_hashes(p.h, row_hashes(p.nrows, seed))
        look = probe
    zh, zl = np.ascontiguousarray(zh, dtype=np.uint64), np.ascontiguousarray(zl, dtype=np.uint64)

    def answer(m, pzh, pzl, plg, pR, res, _ctx):
        try:
            a = [np.ctypeslib.as_array(x, shape=(m,)).copy() for x in (pzh, pzl, plg, pR)]
            np.ctypeslib.as_array(res, shape=(m,))[:] = np.asarray(look(a[0], a[1], a[2], a[3]), dtype=np.int32)
            return 0
        except Exception:                 # reported to the search, which stops with an error
            return 1

    L = _lib.lib()
    native = None
    if probe_fn is not None:
        cb, ctx = probe_fn, probe_ctx
    elif probe is None:
        # the device table answers each wave natively (pinned staging, no interpreter in the loop)
        st = ctypes.c_int(0)
        native = L.tg_tab_probe_create(table.handle, max(1, int(wave)), ctypes.byref(st))
        if not native:
            _lib.check(st.value)
        cb, ctx = PROBE_FN(("tg_tab_probe", L)), native
    else:
        cb, ctx = PROBE_FN(answer), None
    stats = np.zeros(8, dtype=np.int64)
    sol = np.zeros(64, dtype=np.int32)
    nsol = np.zeros(1, dtype=np.int32)
    ptr = lambda a: a.ctypes.data if a.size else None
    try:
        for K in range(start, kmax + 1):
            check_threshold(K)
            t0 = time.time()
            r = L.tg_search(W, n, p.nrows, wmax, ptr(col), ptr(lg), ptr(zh), ptr(zl), ptr(row_start), ptr(row_cols),
                            ptr(col_start), ptr(col_rows), ptr(rank_a), ptr(anch), len(anch), K, k_table, int(wave),
                            cb, ctx, ptr(ex_start) if ex_start is not None else None,
                            ptr(ex_cols) if ex_cols is not None else None, cover_mode, int(threads), float(time_limit),
                            stats.ctypes.data, sol.ctypes.data, nsol.ctypes.data)
            if r < 0:
                _lib.check(r)
            status = {1: "found", 0: "exhausted", 2: "timeout"}[r]
            s = sorted(int(x) for x in sol[:int(nsol[0])]) if r == 1 else []
            best = len(s) if r == 1 else None
            rec = {"K": K, "status": status, "best": best, "nodes": [int(stats[0])], "lookups": int(stats[1]),
                   "hits": int(stats[2]), "false_hits": int(stats[3]), "waves": int(stats[4]),
                   "seconds": time.time() - t0, "tasks": 0, "cover_pruned": int(stats[5]),
                   "nsol_recorded": 1 if r == 1 else 0, "nsol_found": 1 if r == 1 else 0,
                   "solutions_complete": False}
            out["runs"].append(rec)
            if log:
                log(f"  K={K}: {status} best={best} nodes={int(stats[0])} lookups={int(stats[1])} "
                    f"false_hits={int(stats[3])} {rec['seconds']:.2f}s")
            if on_run:
                on_run(rec)
            if r == 2:
                break
            if r == 1:
                syn, lgx = p.check(s)
                assert syn == 0 and lgx != 0 and len(set(s)) == len(s), "reported solution failed verification"
                out["distance"] = best
                out["solutions"] = [tuple(s)]
                out["lower_bound"] = best
                break
            out["lower_bound"] = K + 1
    finally:
        if native:
            L.tg_tab_probe_free(native)
        if table is not None:
            table.free()
    return out
