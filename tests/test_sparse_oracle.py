"""Sparse Rank DP host driver (Trellis, Sweep, query) with the numpy oracle tables, against the
reference's own outputs: slots and masks, per-cut tables, query values and valid witnesses."""
import itertools

import numpy as np

from helpers import golden, sha, unhex
from oracle.sparse import NumpyTables, bound
from tropidist_gb300 import sparse_dp, synth
from tropidist_gb300.problem import Problem


def _problem(case):
    return Problem("rand", case["m"], case["k"], case["h"], case["l"])


def check_witness(p, cols, value, obs=None):
    s = lg = 0
    for j in cols:
        s ^= p.h[j]
        lg ^= p.l[j]
    assert s == 0 and len(cols) == value == len(set(cols))
    assert ((lg >> obs) & 1) if obs is not None else lg != 0


def test_trellis_matches_reference():
    for case in golden("sparse_random.json"):
        tr = sparse_dp.Trellis.for_query(_problem(case), case["obs"], case["order"])
        assert tr.feasible == case["feasible"]
        if tr.feasible:
            assert tr.nslots == case["nslots"] and tr.slot == case["slot"]
            assert tr.tmask == case["tmask"] and tr.col == case["col"]


def test_query_values_with_oracle_tables():
    checked = 0
    for case in golden("sparse_random.json"):
        if not case["feasible"]:
            continue
        p = _problem(case)
        tr = sparse_dp.Trellis.for_query(p, case["obs"], case["order"])
        for run in case["runs"]:
            r = sparse_dp.query(tr, run["K"], mode=run["mode"], split=run["split"], use_h=run["use_h"],
                                backend=NumpyTables(tr))
            assert r["value"] == run["value"], run
            assert r["peak_states"] == run["peak_states"], run
            if run["value"] is not None:
                check_witness(p, r["witness"], run["value"], case["obs"])
            checked += 1
    assert checked > 1000


def test_tables_at_every_cut_match_reference():
    for case in golden("sparse_tables.json"):
        p = Problem("t", case["nrows"], 1, unhex(case["h"]), unhex(case["l"]))
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        sw = sparse_dp.Sweep(tr, +1 if case["forward"] else -1, case["K"], case["K"], use_h=case["use_h"], every=1,
                             backend=NumpyTables(tr))
        sw.run()
        assert sw.counts == case["counts"]
        for c, (n, hk, hv) in case["tables"].items():
            keys, vals = sw.ckpt[int(c)]
            assert keys.size == n and sha(keys) == hk and sha(vals) == hv, c


def test_lookahead_is_admissible():
    """The bound never exceeds the exact remaining cost (the untruncated sweep from the other side)."""
    p = synth.dense_small(3)
    tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
    for fwd in (True, False):
        exact = sparse_dp.Sweep(tr, -1 if fwd else +1, 40, 40, use_h=False, every=1, backend=NumpyTables(tr))
        exact.run()
        hd = tr.bound_data(fwd)
        for c in range(0, tr.N + 1, 7):
            keys, vals = exact.ckpt[c]
            h = bound(keys ^ np.uint64(tr.tmask[c]), tr.tmask[c], hd[c])
            assert (h <= vals.astype(np.int64)).all(), (fwd, c)


def brute(p, obs, weights=None):
    best = None
    for w in range(1, p.ncols + 1):
        if weights is None and best is not None:
            break
        for cols in itertools.combinations(range(p.ncols), w):
            s = lg = 0
            for j in cols:
                s ^= p.h[j]
                lg ^= p.l[j]
            if s == 0 and (lg >> obs) & 1:
                c = w if weights is None else sum(weights[j] for j in cols)
                best = c if best is None else min(best, c)
    return best


def test_weighted_columns_against_brute_force():
    import random
    rng = random.Random(17)
    for _ in range(40):
        n, m = rng.randint(2, 10), rng.randint(1, 6)
        h = [sum(1 << r for r in range(m) if rng.random() < 0.35) for _ in range(n)]
        l = [rng.randrange(0, 2) for _ in range(n)]
        wts = [rng.randint(1, 3) for _ in range(n)]
        p = Problem("w", m, 1, h, l, weights=wts)
        order = list(range(n))
        rng.shuffle(order)
        tr = sparse_dp.Trellis.for_query(p, 0, order)
        truth = brute(p, 0, wts)
        if not tr.feasible:
            assert truth is None
            continue
        K = sum(wts) + 1
        for mode in ("forward", "mitm"):
            r = sparse_dp.query(tr, K, mode=mode, backend=NumpyTables(tr))
            assert r["value"] == truth, (mode, r["value"], truth)
            if truth is not None:
                assert sum(wts[j] for j in r["witness"]) == truth


def test_bound_data_host_routine_matches_restatement():
    """The library's host routine for the lookahead classes equals the numpy restatement of
    cdist/sparse_dp.py:148-192 cut for cut, in both directions."""
    from tropidist_gb300 import sparse_dp, synth
    for seed, rounds, checks, n in [(0, 6, 12, 600), (1, 8, 16, 1500)]:
        p = synth.circuit_dem(seed=seed, rounds=rounds, checks=checks, ncols=n)
        tr = sparse_dp.Trellis.for_query(p, 0, sparse_dp.default_order(p))
        for fwd in (True, False):
            a, b = tr.bound_data(fwd), tr._bound_data_py(fwd)
            assert len(a) == len(b)
            for x, y in zip(a, b):
                assert [int(v) for v in x[0]] == [int(v) for v in y[0]]
                assert [int(v) for v in x[1]] == [int(v) for v in y[1]]
                assert int(x[2]) == int(y[2])


def test_trellis_cut_data_matches_plain_loops():
    """The per-cut data of Trellis (built with array operations) against plain per-row loops:
    active rows (start < c <= end), slot masks, widths, target masks, slot masks per position."""
    from tropidist_gb300 import sparse_dp, synth
    for p in (synth.circuit_dem(seed=2, rounds=10, checks=24, ncols=5000), synth.dense_small(1)):
        order = sparse_dp.default_order(p)
        tr = sparse_dp.Trellis.for_query(p, 0, order)
        assert tr.feasible
        N, nr = tr.N, len(tr.rows)
        act = [[r for r in range(nr) if tr.start[r] < c <= tr.end[r]] for c in range(N + 1)]
        assert tr.active_rows == act
        assert tr.active == [sum(1 << tr.slot[r] for r in a) for a in act]
        assert tr.width == [len(a) for a in act]
        assert tr.tmask == [(1 << tr.slot[tr.L]) if tr.L in a else 0 for a in act]
        col = [0] * N
        for r, row in enumerate(tr.rows):
            x = row
            while x:
                low = x & -x
                col[low.bit_length() - 1] |= 1 << tr.slot[r]
                x ^= low
        assert tr.col == col


def test_c_port_tables_match_reference():
    """oracle/sparse_port.c (the timed CPU baseline of the sparse sweep) behind the backend
    interface: the reference's query values and peak states, and its tables at every cut."""
    from oracle.sparse import CPortTables
    checked = 0
    for case in golden("sparse_random.json"):
        if not case["feasible"]:
            continue
        p = _problem(case)
        tr = sparse_dp.Trellis.for_query(p, case["obs"], case["order"])
        for run in case["runs"]:
            r = sparse_dp.query(tr, run["K"], mode=run["mode"], split=run["split"], use_h=run["use_h"],
                                backend=CPortTables(tr))
            assert r["value"] == run["value"], run
            assert r["peak_states"] == run["peak_states"], run
            if run["value"] is not None:
                check_witness(p, r["witness"], run["value"], case["obs"])
            checked += 1
    assert checked > 1000
    for case in golden("sparse_tables.json"):
        p = Problem("t", case["nrows"], 1, unhex(case["h"]), unhex(case["l"]))
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        sw = sparse_dp.Sweep(tr, +1 if case["forward"] else -1, case["K"], case["K"], use_h=case["use_h"], every=1,
                             backend=CPortTables(tr))
        sw.run()
        assert sw.counts == case["counts"]
        for c, (n, hk, hv) in case["tables"].items():
            keys, vals = CPortTables.arrays(sw.ckpt[int(c)])
            assert keys.size == n and sha(keys) == hk and sha(vals) == hv, c


def test_c_port_weighted_columns_match_numpy():
    """With column weights (no reference caller) the C port's tables equal the numpy restatement's."""
    import random
    from oracle.sparse import CPortTables
    rng = random.Random(5)
    for t in range(30):
        p = synth.banded(20, 40, 6, 3, 1, seed=t)
        p.weights = [rng.randint(1, 3) for _ in range(p.ncols)]
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        if not tr.feasible:
            continue
        for K in (4, 7):
            a = sparse_dp.query(tr, K, backend=NumpyTables(tr), witness=False)
            b = sparse_dp.query(tr, K, backend=CPortTables(tr), witness=False)
            assert a["value"] == b["value"] and a["peak_states"] == b["peak_states"]


def interleaved(copies, seed=0, m=60, n=120, window=12):
    """`copies` independent banded problems with their columns interleaved and only the first one
    carrying the logical row: a trellis as wide as all of them together (beyond one machine word
    for 5 or more copies) whose distance is the first problem's."""
    parts = [synth.banded(m, n, window, 3, 1, seed=seed + k) for k in range(copies)]
    h, l = [], []
    for j in range(n):
        for k, q in enumerate(parts):
            h.append(q.h[j] << (k * m))
            l.append(q.l[j] if k == 0 else 0)
    return Problem("interleaved x%d" % copies, m * copies, 1, h, l), parts[0]


def test_wide_oracle_matches_numpy_tables():
    """The multi-word restatement gives NumpyTables' tables at every cut and its query values on
    one-word states (the reference's own golden tables included)."""
    from oracle.sparse_wide import WideTables
    for case in golden("sparse_tables.json"):
        p = Problem("t", case["nrows"], 1, unhex(case["h"]), unhex(case["l"]))
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        be = WideTables(tr, words=2)
        sw = sparse_dp.Sweep(tr, +1 if case["forward"] else -1, case["K"], case["K"], use_h=case["use_h"], every=1,
                             backend=be)
        sw.run()
        assert sw.counts == case["counts"]
        for c, (n, hk, hv) in case["tables"].items():
            keys, vals = be.arrays(sw.ckpt[int(c)])
            assert len(keys) == n and sha(np.array(keys, dtype=np.uint64)) == hk and sha(vals) == hv, c


def test_wide_trellis_queries():
    """Trellises of more than 64 row slots (interleaved copies): lookahead classes of every cut
    against plain per-row loops, and the multi-word query's value equal to the first copy's own
    (one-word) query, with a valid witness."""
    from oracle.sparse_wide import WideTables
    for copies, seed in ((8, 0), (10, 3)):
        p, first = interleaved(copies, seed)
        order = list(range(p.ncols))
        tr = sparse_dp.Trellis.for_query(p, 0, order)
        assert tr.nslots > 64 and tr.words >= 2
        for fwd in (True, False):
            ncls, masks, wts, extra = tr.bound_raw(fwd)
            slow = tr._bound_data_py(fwd)
            for c in range(tr.N + 1):
                got = tuple(sum(int(masks[c, k, q]) << (64 * q) for q in range(tr.words)) for k in range(ncls[c]))
                assert got == slow[c][0] and tuple(wts[c, :ncls[c]]) == slow[c][1] and extra[c] == slow[c][2]
        t1 = sparse_dp.Trellis.for_query(first, 0, list(range(first.ncols)))
        for K in (3, 5):
            want = sparse_dp.query(t1, K, backend=NumpyTables(t1))
            got = sparse_dp.query(tr, K, backend=WideTables(tr))
            assert got["value"] == want["value"]
            if got["value"] is not None:
                check_witness(p, got["witness"], got["value"], 0)
