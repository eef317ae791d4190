"""Sparse Rank DP on device tables of multi-word states (more than 64 row slots, beyond the
reference's limit), against the multi-word oracle restatement and the reference's own results."""
import random

import numpy as np
import pytest

from helpers import golden, unhex
from oracle.sparse import NumpyTables
from oracle.sparse_wide import WideTables
from test_sparse_oracle import check_witness, interleaved

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _tables(be, tab):
    keys, vals = be.arrays(tab)
    return list(keys), np.asarray(vals).tolist()


def test_wide_tables_at_every_cut_match_oracle():
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.sparse_tables import WideGpuTables
    for copies, seed in ((8, 0), (10, 3)):
        p, _ = interleaved(copies, seed)
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        assert tr.words >= 2
        for direction, K, use_h in ((+1, 4, True), (-1, 4, True), (+1, 3, False)):
            sweeps = {}
            for name, be in (("gpu", WideGpuTables(tr)), ("oracle", WideTables(tr))):
                sw = sparse_dp.Sweep(tr, direction, K, K, use_h=use_h, every=1, backend=be)
                sw.run()
                sweeps[name] = sw
            g, o = sweeps["gpu"], sweeps["oracle"]
            assert g.counts == o.counts and g.peak == o.peak
            for c in range(0, tr.N + 1, 7):
                assert _tables(g.be, g.ckpt[c]) == _tables(o.be, o.ckpt[c]), (copies, direction, c)


def test_wide_frontier_sweeps_match_oracle_cut_by_cut():
    """Forward frontier sweeps with falling caps: every table and changed set equal the oracle's."""
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.sparse_tables import WideGpuTables
    rng = random.Random(9)
    p, _ = interleaved(8, 5)
    tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
    K = 5
    caps = sorted((rng.randint(1, K) for _ in range(tr.N + 1)), reverse=True)
    rec = {}
    for name, be in (("gpu", WideGpuTables(tr)), ("oracle", WideTables(tr))):
        sw = sparse_dp.Sweep(tr, +1, K, use_h=True, every=1, frontier=True, backend=be, caps=caps)
        out = []

        def on_cut(c, tab, ch, extra, sw=sw, out=out):
            part = _tables(sw.be, ch) if ch is not None else None
            out.append((c, _tables(sw.be, tab), part))
            return False
        sw.run(on_cut=on_cut)
        rec[name] = out
    assert rec["gpu"] == rec["oracle"]


@pytest.mark.parametrize("words", [1, 2, 8])
def test_wide_tables_reproduce_reference_queries(words):
    """One-word problems through the multi-word device tables: the reference's values and peaks."""
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.problem import Problem
    from tropidist_gb300.sparse_tables import WideGpuTables
    checked = 0
    for case in golden("sparse_random.json")[::4]:
        if not case["feasible"]:
            continue
        p = Problem("rand", case["m"], case["k"], case["h"], case["l"])
        tr = sparse_dp.Trellis.for_query(p, case["obs"], case["order"])
        for run in case["runs"][::5]:
            r = sparse_dp.query(tr, run["K"], mode=run["mode"], split=run["split"], use_h=run["use_h"],
                                backend=WideGpuTables(tr, words=words))
            assert r["value"] == run["value"] and r["peak_states"] == run["peak_states"], run
            if run["value"] is not None:
                check_witness(p, r["witness"], run["value"], case["obs"])
            checked += 1
    assert checked > 50


def test_wide_queries_and_distance():
    """Trellises of more than 64 slots: the query value equals the first copy's own and the witness
    is valid; distance() picks the wide tables by itself."""
    from tropidist_gb300 import sparse_dp
    for copies, seed in ((8, 1), (9, 2)):
        p, first = interleaved(copies, seed)
        tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
        t1 = sparse_dp.Trellis.for_query(first, 0, list(range(first.ncols)))
        for K, mode in ((4, "mitm"), (6, "mitm"), (4, "forward")):
            want = sparse_dp.query(t1, K, mode=mode, backend=NumpyTables(t1))
            got = sparse_dp.query(tr, K, mode=mode)
            assert got["backend"] == "gpu" and got["value"] == want["value"], (copies, K, mode)
            if got["value"] is not None:
                check_witness(p, got["witness"], got["value"], 0)
        d = sparse_dp.distance(p, order=list(range(p.ncols)), kmax=12)
        d1 = sparse_dp.distance(first, order=list(range(first.ncols)), kmax=12)
        assert d["distance"] == d1["distance"]


def test_wide_walk_grows_its_tables_and_arena():
    """Device walks started with tables and an arena far too small run their legs again with more
    room: the same counts, peaks and kept tables as the oracle's step-by-step sweep."""
    from tropidist_gb300 import sparse_dp
    from tropidist_gb300.sparse_tables import WideGpuTables
    p, _ = interleaved(8, 4)
    tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
    # capacity 1: every leg runs again; 64: the one-block walk hands over to the separate launches
    # and back many times
    for direction, cap0 in ((+1, 1), (-1, 1), (+1, 64), (-1, 64)):
        be = WideGpuTables(tr)
        be._walk_cap, be._arena_guess = cap0, 1
        sw = sparse_dp.Sweep(tr, direction, 5, 5, every=3, backend=be)
        sw.run()
        assert be._walk_cap >= 64
        ref = sparse_dp.Sweep(tr, direction, 5, 5, every=3, backend=WideTables(tr))
        ref.run(on_cut=lambda *a: False)
        assert sw.counts == ref.counts and sw.peak == ref.peak
        for c, t in sw.ckpt.items():
            assert _tables(be, t) == _tables(ref.be, ref.ckpt[c]), (direction, c)


@pytest.mark.parametrize("limit", [0, 64, None])
def test_wide_meet_by_walks_equals_step_by_step(limit):
    """The meet in the middle run as device walks (joins inside the walk, frontier truncation)
    gives the value, peak, join counts and a valid witness as the step-by-step meet on the oracle
    tables: with separate launches only (limit 0), the one-block walk handing over at 32 states,
    and the default."""
    from tropidist_gb300 import _lib, sparse_dp
    L = _lib.lib()
    old = L.tg_spw_set_small_limit(-1)
    try:
        if limit is not None:
            L.tg_spw_set_small_limit(limit)
        for copies, seed in ((8, 6), (9, 7)):
            p, _ = interleaved(copies, seed)
            tr = sparse_dp.Trellis.for_query(p, 0, list(range(p.ncols)))
            for K in (3, 5):
                got = sparse_dp.query(tr, K, mode="mitm")
                want = sparse_dp.query(tr, K, mode="mitm", backend=WideTables(tr))
                assert got["value"] == want["value"] and got["peak_states"] == want["peak_states"], (copies, K)
                assert got["changed_counts"] == want["changed_counts"], (copies, K)
                if got["value"] is not None:
                    check_witness(p, got["witness"], got["value"], 0)
    finally:
        L.tg_spw_set_small_limit(old)


@pytest.mark.parametrize("shape", [(6, 80, 1200), (4, 150, 1200)])
def test_wide_weighted_circuits_match_oracle(shape):
    """Circuit-style problems with column weights {1, 2, 3} and more than 64 row slots (the
    structure of the problem as written, at a size the oracle finishes in about a second): the
    device query's value, peak and changed counts equal the multi-word oracle's, its witness has
    the value as its weight, and a backward sweep's tables equal the oracle's cut by cut."""
    from tropidist_gb300 import sparse_dp, synth
    from tropidist_gb300.sparse_tables import WideGpuTables
    rounds, checks, ncols = shape
    p = synth.circuit_dem(seed=1, rounds=rounds, checks=checks, ncols=ncols)
    tr = sparse_dp.Trellis.for_query(p, 0, sparse_dp.default_order(p))
    assert tr.nslots > 64 and len(set(p.weights)) == 3
    for K in (4, 6):
        got = sparse_dp.query(tr, K, mode="mitm")
        want = sparse_dp.query(tr, K, mode="mitm", backend=WideTables(tr))
        assert got["backend"] == "gpu"
        assert got["value"] == want["value"] and got["peak_states"] == want["peak_states"], K
        assert got["changed_counts"] == want["changed_counts"], K
        if got["value"] is not None:
            cols = got["witness"]
            s = lg = 0
            for j in cols:
                s ^= p.h[j]
                lg ^= p.l[j]
            assert s == 0 and lg & 1 and sum(p.weights[j] for j in cols) == got["value"]
    g = sparse_dp.Sweep(tr, -1, 6, 6, every=5, backend=WideGpuTables(tr))
    g.run()
    o = sparse_dp.Sweep(tr, -1, 6, 6, every=5, backend=WideTables(tr))
    o.run(on_cut=lambda *a: False)
    assert g.counts == o.counts and g.peak == o.peak
    for c, t in g.ckpt.items():
        assert _tables(g.be, t) == _tables(o.be, o.ckpt[c]), c
